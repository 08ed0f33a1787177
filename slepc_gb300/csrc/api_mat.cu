// api_mat.cu -- PETSc's matrix and vector assembly calls for sequential AIJ (petscmat.h, petscvec.h): MatSetSizes,
// MatSetValue(s), MatAssemblyBegin/End, MatSetOption, MatZeroEntries, MatScale, MatShift, and VecCreate/SetSizes/
// SetValue(s)/PlaceArray/DuplicateVecs.  The reference's examples build their operators this way
// (src/eps/tutorials/ex2.c:54-66, src/eps/tests/test1.c:38-54).
//
// Host code only.  MatSetValue(s) append entries; MatAssemblyEnd orders them by row (counting sort) and by column
// within a row (stable), combines repeated positions in call order -- INSERT_VALUES replaces, ADD_VALUES adds -- and
// builds the CSR arrays the Mat then owns.  Entries of an earlier assembly take part as inserted values, so values can
// be changed and nonzeros added between assemblies.  Any change drops the device copy and the cached norm and bumps
// the matrix state, which makes an EPS set up on the matrix set up again at its next solve.
#include <algorithm>
#include <cstring>
#include <vector>

#include "internal.h"

namespace {

// the Mat's CSR arrays become library-owned (MatCreateSeqAIJWithArrays matrices keep the caller's arrays until then)
void own_arrays(Mat A) {
  if (A->ai == A->own_i.data() && !A->own_i.empty()) return;
  if (A->ai) {
    A->own_i.assign(A->ai, A->ai + A->m + 1);
    A->own_j.assign(A->aj, A->aj + A->nnz);
    A->own_a.assign(A->aa, A->aa + A->nnz);
  } else {
    A->own_i.assign(A->m + 1, 0);
    A->own_j.clear();
    A->own_a.clear();
  }
  A->ai = A->own_i.data();
  A->aj = A->own_j.data();
  A->aa = A->own_a.data();
}

// the values changed: device copies and the cached norm go; solvers set up on the matrix set up again
void values_changed(Mat A) {
  A->d_rp.release();
  A->d_ci.release();
  A->d_va.release();
  A->d_va2.release();
  A->d_va32.release();
  A->d_seg_row.release();
  A->d_seg_beg.release();
  A->d_seg_end.release();
  A->d_lrow.release();
  A->d_lfirst.release();
  A->n_long = A->n_seg = 0;
  A->device_ready = 0;
  A->norm_inf = -1.0;
  A->state++;
}

PetscErrorCode check_aij(Mat A) {
  KSG_CHECK(A, PETSC_ERR_ARG_NULL, "Null Mat");
  KSG_CHECK(!A->dense, PETSC_ERR_SUP, "Only sequential AIJ matrices are assembled here");
  KSG_CHECK(A->sized || !A->empty, PETSC_ERR_ORDER, "Must call MatSetSizes() first");
  return 0;
}

}  // namespace

extern "C" PetscErrorCode MatSetSizes(Mat A, PetscInt m, PetscInt n, PetscInt M, PetscInt N) {
  KSG_CHECK(A, PETSC_ERR_ARG_NULL, "Null Mat");
  KSG_CHECK(A->empty && !A->sized, PETSC_ERR_ARG_WRONGSTATE, "The sizes of this Mat are already set");
  KSG_CHECK(!(m == PETSC_DECIDE && M == PETSC_DECIDE) && !(n == PETSC_DECIDE && N == PETSC_DECIDE),
            PETSC_ERR_ARG_OUTOFRANGE, "Either the local or the global size must be given");
  const PetscInt rows = M != PETSC_DECIDE ? M : m, cols = N != PETSC_DECIDE ? N : n;
  // one process: the local size is the global size
  KSG_CHECK(m == PETSC_DECIDE || m == rows, PETSC_ERR_ARG_INCOMP, "Local row size %d differs from the global %d",
            (int)m, (int)rows);
  KSG_CHECK(n == PETSC_DECIDE || n == cols, PETSC_ERR_ARG_INCOMP, "Local column size %d differs from the global %d",
            (int)n, (int)cols);
  KSG_CHECK(rows >= 0 && cols >= 0, PETSC_ERR_ARG_OUTOFRANGE, "Negative size");
  A->m = rows;
  A->n = cols;
  A->sized = 1;
  return 0;
}

extern "C" PetscErrorCode MatSetUp(Mat A) { return check_aij(A); }

extern "C" PetscErrorCode MatSeqAIJSetPreallocation(Mat A, PetscInt, const PetscInt[]) {
  return check_aij(A);  // storage grows as values arrive
}

extern "C" PetscErrorCode MatGetOwnershipRange(Mat A, PetscInt *rstart, PetscInt *rend) {
  KSG_CHECK(A, PETSC_ERR_ARG_NULL, "Null Mat");
  if (rstart) *rstart = 0;
  if (rend) *rend = A->m;
  return 0;
}

extern "C" PetscErrorCode MatGetLocalSize(Mat A, PetscInt *m, PetscInt *n) {
  KSG_CHECK(A, PETSC_ERR_ARG_NULL, "Null Mat");
  if (m) *m = A->m;
  if (n) *n = A->n;
  return 0;
}

// MatSetValues: v is m x n, row-major; a negative row or column index skips its entries
extern "C" PetscErrorCode MatSetValues(Mat A, PetscInt m, const PetscInt idxm[], PetscInt n, const PetscInt idxn[],
                                       const PetscScalar v[], InsertMode mode) {
  KSG_TRY(check_aij(A));
  KSG_CHECK(mode == INSERT_VALUES || mode == ADD_VALUES, PETSC_ERR_SUP, "Only INSERT_VALUES and ADD_VALUES");
  KSG_CHECK((m == 0 || idxm) && (n == 0 || idxn) && (m * n == 0 || v), PETSC_ERR_ARG_NULL, "Null argument");
  for (PetscInt r = 0; r < m; ++r) {
    const PetscInt i = idxm[r];
    if (i < 0) continue;
    KSG_CHECK(i < A->m, PETSC_ERR_ARG_OUTOFRANGE, "Row too large: row %d max %d", (int)i, A->m - 1);
    for (PetscInt c = 0; c < n; ++c) {
      const PetscInt j = idxn[c];
      if (j < 0) continue;
      KSG_CHECK(j < A->n, PETSC_ERR_ARG_OUTOFRANGE, "Column too large: col %d max %d", (int)j, A->n - 1);
      A->pending.push_back({(int)i, (int)j, v[r * n + c], mode == ADD_VALUES});
    }
  }
  return 0;
}

extern "C" PetscErrorCode MatSetValue(Mat A, PetscInt i, PetscInt j, PetscScalar v, InsertMode mode) {
  return MatSetValues(A, 1, &i, 1, &j, &v, mode);
}

extern "C" PetscErrorCode MatAssemblyBegin(Mat A, MatAssemblyType) { return check_aij(A); }

// MatAssemblyEnd: the CSR arrays from the earlier assembly (as inserted values) and the pending entries
extern "C" PetscErrorCode MatAssemblyEnd(Mat A, MatAssemblyType) {
  KSG_TRY(check_aij(A));
  if (A->pending.empty() && !A->empty) return 0;
  const int m = A->m;
  std::vector<MatEntry> all;
  all.reserve((size_t)A->nnz + A->pending.size());
  if (!A->empty)
    for (int r = 0; r < m; ++r)
      for (PetscInt p = A->ai[r]; p < A->ai[r + 1]; ++p) all.push_back({r, (int)A->aj[p], A->aa[p], 0});
  all.insert(all.end(), A->pending.begin(), A->pending.end());
  std::vector<MatEntry>().swap(A->pending);
  // by row, keeping call order (counting sort), then by column within the row (stable)
  std::vector<size_t> start(m + 1, 0);
  for (const MatEntry &e : all) start[e.row + 1]++;
  for (int r = 0; r < m; ++r) start[r + 1] += start[r];
  std::vector<MatEntry> byrow(all.size());
  {
    std::vector<size_t> fill(start.begin(), start.end() - 1);
    for (const MatEntry &e : all) byrow[fill[e.row]++] = e;
  }
  std::vector<PetscInt> ai(m + 1, 0), aj;
  std::vector<double> aa;
  aj.reserve(byrow.size());
  aa.reserve(byrow.size());
  for (int r = 0; r < m; ++r) {
    auto b = byrow.begin() + start[r], e = byrow.begin() + start[r + 1];
    std::stable_sort(b, e, [](const MatEntry &x, const MatEntry &y) { return x.col < y.col; });
    for (auto it = b; it != e;) {
      double v = 0.0;
      const int col = it->col;
      for (; it != e && it->col == col; ++it) v = it->add ? v + it->v : it->v;
      aj.push_back(col);
      aa.push_back(v);
    }
    ai[r + 1] = (PetscInt)aj.size();
  }
  A->own_i.swap(ai);
  A->own_j.swap(aj);
  A->own_a.swap(aa);
  A->ai = A->own_i.data();
  A->aj = A->own_j.data();
  A->aa = A->own_a.data();
  A->nnz = (long long)A->own_j.size();
  A->empty = 0;
  values_changed(A);
  return 0;
}

extern "C" PetscErrorCode MatAssembled(Mat A, PetscBool *assembled) {
  KSG_CHECK(A && assembled, PETSC_ERR_ARG_NULL, "Null argument");
  *assembled = (!A->empty && A->pending.empty()) ? PETSC_TRUE : PETSC_FALSE;
  return 0;
}

extern "C" PetscErrorCode MatSetOption(Mat A, MatOption, PetscBool) {
  KSG_CHECK(A, PETSC_ERR_ARG_NULL, "Null Mat");
  return 0;  // hints (symmetry, nonzero-pattern policies) that do not change the values
}

extern "C" PetscErrorCode MatZeroEntries(Mat A) {
  KSG_CHECK(A, PETSC_ERR_ARG_NULL, "Null Mat");
  if (A->dense) {
    for (int c = 0; c < A->n; ++c)
      for (int r = 0; r < A->m; ++r) A->data[r + (size_t)c * A->lda] = 0.0;
  } else if (!A->empty) {
    own_arrays(A);
    std::fill(A->own_a.begin(), A->own_a.end(), 0.0);
  }
  values_changed(A);
  return 0;
}

extern "C" PetscErrorCode MatScale(Mat A, PetscScalar a) {
  KSG_CHECK(A, PETSC_ERR_ARG_NULL, "Null Mat");
  KSG_CHECK(!A->empty, PETSC_ERR_ARG_WRONGSTATE, "Not for unassembled matrix");
  if (A->dense) {
    for (int c = 0; c < A->n; ++c)
      for (int r = 0; r < A->m; ++r) A->data[r + (size_t)c * A->lda] *= a;
  } else {
    own_arrays(A);
    for (double &x : A->own_a) x *= a;
  }
  values_changed(A);
  return 0;
}

// MatShift: A + a I (diagonal entries missing from the pattern are added)
extern "C" PetscErrorCode MatShift(Mat A, PetscScalar a) {
  KSG_CHECK(A, PETSC_ERR_ARG_NULL, "Null Mat");
  KSG_CHECK(!A->empty, PETSC_ERR_ARG_WRONGSTATE, "Not for unassembled matrix");
  KSG_CHECK(A->m == A->n, PETSC_ERR_ARG_WRONG, "MatShift needs a square matrix");
  if (A->dense) {
    for (int r = 0; r < A->m; ++r) A->data[r + (size_t)r * A->lda] += a;
    values_changed(A);
    return 0;
  }
  own_arrays(A);
  for (int r = 0; r < A->m; ++r) A->pending.push_back({r, r, a, 1});
  return MatAssemblyEnd(A, MAT_FINAL_ASSEMBLY);
}

// ---------------------------------------------------------------------------------------------------------------
// Vec
// ---------------------------------------------------------------------------------------------------------------
extern "C" PetscErrorCode VecCreate(MPI_Comm, Vec *v) {
  KSG_CHECK(v, PETSC_ERR_ARG_NULL, "Null Vec pointer");
  *v = new _p_Vec();
  (*v)->n = -1;  // sizes not set
  return 0;
}

extern "C" PetscErrorCode VecSetSizes(Vec v, PetscInt n, PetscInt N) {
  KSG_CHECK(v, PETSC_ERR_ARG_NULL, "Null Vec");
  KSG_CHECK(v->n < 0, PETSC_ERR_ARG_WRONGSTATE, "The size of this Vec is already set");
  const PetscInt size = N != PETSC_DECIDE ? N : n;
  KSG_CHECK(size >= 0, PETSC_ERR_ARG_OUTOFRANGE, "Either the local or the global size must be given");
  KSG_CHECK(n == PETSC_DECIDE || n == size, PETSC_ERR_ARG_INCOMP, "Local size %d differs from the global %d", (int)n,
            (int)size);
  v->n = size;
  v->own.assign(size > 0 ? size : 1, 0.0);
  v->a = v->own.data();
  return 0;
}

extern "C" PetscErrorCode VecSetFromOptions(Vec v) {
  KSG_CHECK(v, PETSC_ERR_ARG_NULL, "Null Vec");
  KSG_CHECK(v->n >= 0, PETSC_ERR_ORDER, "Must call VecSetSizes() first");
  return 0;
}

extern "C" PetscErrorCode VecSetValues(Vec v, PetscInt ni, const PetscInt ix[], const PetscScalar y[],
                                       InsertMode mode) {
  KSG_CHECK(v && (ni == 0 || (ix && y)), PETSC_ERR_ARG_NULL, "Null argument");
  KSG_CHECK(v->n >= 0, PETSC_ERR_ORDER, "Must call VecSetSizes() first");
  KSG_CHECK(mode == INSERT_VALUES || mode == ADD_VALUES, PETSC_ERR_SUP, "Only INSERT_VALUES and ADD_VALUES");
  for (PetscInt k = 0; k < ni; ++k) {
    const PetscInt i = ix[k];
    if (i < 0) continue;
    KSG_CHECK(i < v->n, PETSC_ERR_ARG_OUTOFRANGE, "Out of range index value %d maximum %d", (int)i, v->n);
    v->a[i] = mode == ADD_VALUES ? v->a[i] + y[k] : y[k];
  }
  return 0;
}

extern "C" PetscErrorCode VecSetValue(Vec v, PetscInt i, PetscScalar y, InsertMode mode) {
  return VecSetValues(v, 1, &i, &y, mode);
}

extern "C" PetscErrorCode VecAssemblyBegin(Vec v) {
  KSG_CHECK(v, PETSC_ERR_ARG_NULL, "Null Vec");
  return 0;  // values are stored as they are set (one process)
}

extern "C" PetscErrorCode VecAssemblyEnd(Vec v) {
  KSG_CHECK(v, PETSC_ERR_ARG_NULL, "Null Vec");
  return 0;
}

extern "C" PetscErrorCode VecZeroEntries(Vec v) {
  KSG_CHECK(v, PETSC_ERR_ARG_NULL, "Null Vec");
  if (v->n > 0) std::memset(v->a, 0, sizeof(double) * v->n);
  return 0;
}

extern "C" PetscErrorCode VecDuplicateVecs(Vec v, PetscInt m, Vec *V[]) {
  KSG_CHECK(v && V, PETSC_ERR_ARG_NULL, "Null argument");
  KSG_CHECK(m > 0, PETSC_ERR_ARG_OUTOFRANGE, "m must be > 0: m = %d", (int)m);
  Vec *arr = new Vec[m];
  for (PetscInt k = 0; k < m; ++k) {
    const PetscErrorCode ierr = VecDuplicate(v, &arr[k]);
    if (ierr) {
      for (PetscInt q = 0; q < k; ++q) VecDestroy(&arr[q]);
      delete[] arr;
      return ierr;
    }
  }
  *V = arr;
  return 0;
}

extern "C" PetscErrorCode VecDestroyVecs(PetscInt m, Vec *V[]) {
  if (!V || !*V) return 0;
  for (PetscInt k = 0; k < m; ++k) VecDestroy(&(*V)[k]);
  delete[] *V;
  *V = nullptr;
  return 0;
}

// VecPlaceArray / VecResetArray: the Vec reads and writes the caller's array until it is reset
extern "C" PetscErrorCode VecPlaceArray(Vec v, const PetscScalar array[]) {
  KSG_CHECK(v, PETSC_ERR_ARG_NULL, "Null Vec");
  KSG_CHECK(!v->placed_from, PETSC_ERR_ARG_WRONGSTATE, "VecPlaceArray() was already called on this vector, "
            "without a call to VecResetArray()");
  v->placed_from = v->a;
  v->a = const_cast<double *>(array);
  return 0;
}

extern "C" PetscErrorCode VecResetArray(Vec v) {
  KSG_CHECK(v, PETSC_ERR_ARG_NULL, "Null Vec");
  if (v->placed_from) {
    v->a = v->placed_from;
    v->placed_from = nullptr;
  }
  return 0;
}

extern "C" PetscErrorCode VecConjugate(Vec v) {
  KSG_CHECK(v, PETSC_ERR_ARG_NULL, "Null Vec");
  return 0;  // real scalars
}

extern "C" PetscErrorCode VecGetOwnershipRange(Vec v, PetscInt *low, PetscInt *high) {
  KSG_CHECK(v, PETSC_ERR_ARG_NULL, "Null Vec");
  if (low) *low = 0;
  if (high) *high = v->n;
  return 0;
}

// ---------------------------------------------------------------------------------------------------------------
// small PETSc utilities the examples use: string compare, MPI on one process, random numbers, orthonormality check
// ---------------------------------------------------------------------------------------------------------------
extern "C" PetscErrorCode PetscStrcmp(const char a[], const char b[], PetscBool *flg) {
  KSG_CHECK(flg, PETSC_ERR_ARG_NULL, "Null argument");
  *flg = ((!a && !b) || (a && b && !std::strcmp(a, b))) ? PETSC_TRUE : PETSC_FALSE;
  return 0;
}

extern "C" int MPI_Comm_rank(MPI_Comm, int *rank) {
  if (rank) *rank = 0;
  return 0;
}

extern "C" int MPI_Comm_size(MPI_Comm, int *size) {
  if (size) *size = 1;
  return 0;
}

struct _p_PetscRandom {
  unsigned long long seed = 0x5EEDULL;
  unsigned long long counter = 0;
  double low = 0.0, width = 1.0;  // PetscRandomSetInterval
};

extern "C" PetscErrorCode PetscRandomCreate(MPI_Comm, PetscRandom *r) {
  KSG_CHECK(r, PETSC_ERR_ARG_NULL, "Null argument");
  *r = new _p_PetscRandom();
  return 0;
}

extern "C" PetscErrorCode PetscRandomSetFromOptions(PetscRandom r) {
  KSG_CHECK(r, PETSC_ERR_ARG_NULL, "Null PetscRandom");
  return 0;
}

extern "C" PetscErrorCode PetscRandomSetSeed(PetscRandom r, unsigned long seed) {
  KSG_CHECK(r, PETSC_ERR_ARG_NULL, "Null PetscRandom");
  r->seed = seed;
  return 0;
}

extern "C" PetscErrorCode PetscRandomSeed(PetscRandom r) {
  KSG_CHECK(r, PETSC_ERR_ARG_NULL, "Null PetscRandom");
  r->counter = 0;  // restart the stream of the current seed
  return 0;
}

// the next value of the stream, uniform in [0, 1) (splitmix64, the top 53 bits)
static double random_next(PetscRandom r) {
  unsigned long long z = r->seed + (++r->counter) * 0x9E3779B97F4A7C15ULL;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  z ^= z >> 31;
  return (double)(z >> 11) * (1.0 / 9007199254740992.0);
}

extern "C" PetscErrorCode PetscRandomGetValue(PetscRandom r, PetscScalar *value) {
  KSG_CHECK(r && value, PETSC_ERR_ARG_NULL, "Null argument");
  *value = r->low + r->width * random_next(r);
  return 0;
}

extern "C" PetscErrorCode PetscRandomGetValueReal(PetscRandom r, PetscReal *value) {
  return PetscRandomGetValue(r, value);
}

extern "C" PetscErrorCode PetscRandomSetInterval(PetscRandom r, PetscScalar low, PetscScalar high) {
  KSG_CHECK(r, PETSC_ERR_ARG_NULL, "Null PetscRandom");
  KSG_CHECK(low < high, PETSC_ERR_ARG_OUTOFRANGE, "only low < high");
  r->low = low;
  r->width = high - low;
  return 0;
}

extern "C" PetscErrorCode PetscStrendswith(const char a[], const char b[], PetscBool *flg) {
  KSG_CHECK(flg, PETSC_ERR_ARG_NULL, "Null argument");
  *flg = PETSC_FALSE;
  if (a && b) {
    const size_t la = std::strlen(a), lb = std::strlen(b);
    *flg = (la >= lb && !std::strcmp(a + la - lb, b)) ? PETSC_TRUE : PETSC_FALSE;
  }
  return 0;
}

extern "C" PetscErrorCode PetscSplitOwnership(MPI_Comm, PetscInt *n, PetscInt *N) {
  KSG_CHECK(n && N, PETSC_ERR_ARG_NULL, "Null argument");
  KSG_CHECK(*n != PETSC_DECIDE || *N != PETSC_DECIDE, PETSC_ERR_ARG_INCOMP, "Both n and N cannot be PETSC_DECIDE");
  if (*n == PETSC_DECIDE) *n = *N;
  if (*N == PETSC_DECIDE) *N = *n;
  KSG_CHECK(*n == *N, PETSC_ERR_ARG_SIZ, "Sum of local lengths %d does not equal global length %d", (int)*n, (int)*N);
  return 0;
}

extern "C" PetscErrorCode PetscRandomDestroy(PetscRandom *r) {
  if (!r || !*r) return 0;
  delete *r;
  *r = nullptr;
  return 0;
}

extern "C" PetscErrorCode VecSetRandom(Vec v, PetscRandom r) {
  KSG_CHECK(v, PETSC_ERR_ARG_NULL, "Null Vec");
  _p_PetscRandom local;
  PetscRandom rr = r ? r : &local;
  for (int i = 0; i < v->n; ++i) v->a[i] = rr->low + rr->width * random_next(rr);
  return 0;
}

// VecCheckOrthonormality (src/sys/vec/vecutil.c): the largest entry of |Y^T B X - I| (host arithmetic)
extern "C" PetscErrorCode VecCheckOrthonormality(Vec x[], PetscInt nx, Vec y[], PetscInt ny, Mat B, PetscViewer,
                                                 PetscReal *lev) {
  KSG_CHECK(x && lev, PETSC_ERR_ARG_NULL, "Null argument");
  if (!y) {
    y = x;
    ny = nx;
  }
  const int n = nx > 0 ? x[0]->n : 0;
  std::vector<double> bx((size_t)n);
  double worst = 0.0;
  for (PetscInt i = 0; i < nx; ++i) {
    KSG_CHECK(x[i] && x[i]->n == n, PETSC_ERR_ARG_SIZ, "Vectors of different sizes");
    const double *xi = x[i]->a;
    if (B) {  // b = B x_i
      KSG_CHECK(!B->empty && !B->dense && B->m == n && B->n == n, PETSC_ERR_ARG_WRONG,
                "B must be an assembled square AIJ matrix of the vectors' size");
      for (int r = 0; r < n; ++r) {
        double s = 0.0;
        for (PetscInt p = B->ai[r]; p < B->ai[r + 1]; ++p) s += B->aa[p] * xi[B->aj[p]];
        bx[r] = s;
      }
      xi = bx.data();
    }
    for (PetscInt j = 0; j < ny; ++j) {
      KSG_CHECK(y[j] && y[j]->n == n, PETSC_ERR_ARG_SIZ, "Vectors of different sizes");
      double d = 0.0;
      for (int r = 0; r < n; ++r) d += y[j]->a[r] * xi[r];
      worst = std::max(worst, std::fabs(d - (i == j ? 1.0 : 0.0)));
    }
  }
  *lev = worst;
  return 0;
}

// MatDuplicate: a library-owned copy (values or zeros); MatDiagonalSet: the diagonal from a Vec
extern "C" PetscErrorCode MatDuplicate(Mat A, MatDuplicateOption op, Mat *B) {
  KSG_CHECK(A && B, PETSC_ERR_ARG_NULL, "Null argument");
  KSG_CHECK(!A->empty, PETSC_ERR_ARG_WRONGSTATE, "Not for unassembled matrix");
  KSG_CHECK(!A->dense, PETSC_ERR_SUP, "MatDuplicate of a dense Mat is not provided");
  Mat C = new _p_Mat();
  C->m = A->m;
  C->n = A->n;
  C->sized = 1;
  C->own_i.assign(A->ai, A->ai + A->m + 1);
  C->own_j.assign(A->aj, A->aj + A->nnz);
  if (op == MAT_COPY_VALUES) C->own_a.assign(A->aa, A->aa + A->nnz);
  else C->own_a.assign((size_t)A->nnz, 0.0);
  C->ai = C->own_i.data();
  C->aj = C->own_j.data();
  C->aa = C->own_a.data();
  C->nnz = A->nnz;
  *B = C;
  return 0;
}

extern "C" PetscErrorCode MatDiagonalSet(Mat A, Vec D, InsertMode mode) {
  KSG_CHECK(A && D, PETSC_ERR_ARG_NULL, "Null argument");
  KSG_CHECK(!A->empty, PETSC_ERR_ARG_WRONGSTATE, "Not for unassembled matrix");
  KSG_CHECK(!A->dense && D->n == std::min(A->m, A->n), PETSC_ERR_ARG_SIZ, "Nonconforming sizes");
  KSG_CHECK(mode == INSERT_VALUES || mode == ADD_VALUES, PETSC_ERR_SUP, "Only INSERT_VALUES and ADD_VALUES");
  own_arrays(A);
  for (int r = 0; r < D->n; ++r) A->pending.push_back({r, r, D->a[r], mode == ADD_VALUES});
  return MatAssemblyEnd(A, MAT_FINAL_ASSEMBLY);
}
