// api_io.cu -- PETSc binary matrix and vector files (PetscViewerBinaryOpen, MatLoad, MatView, VecLoad, VecView).
//
// The reference's tutorials read their operators this way (src/eps/tutorials/ex4.c:45-49, ex7.c:52, ex31.c:551-562),
// and its data files (share/slepc/datafiles/matrices/*.petsc) use PETSc's binary format: every item big-endian,
//   matrix: int32 MAT_FILE_CLASSID, rows, columns, nonzeros; int32 row lengths[rows]; int32 column indices[nnz];
//           float64 values[nnz];
//   vector: int32 VEC_FILE_CLASSID, length; float64 values[length].
// Items are assembled byte by byte, so the files read and write the same on little- and big-endian hosts.  A loaded
// matrix owns its CSR arrays; everything else about it (device upload on first solve, MatMult, MatDestroy) is the
// same as for MatCreateSeqAIJWithArrays.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "internal.h"

struct _p_PetscViewer {
  FILE *f = nullptr;
  PetscFileMode mode = FILE_MODE_READ;
  std::string name;
};

namespace {

void put_be(std::vector<unsigned char> &out, unsigned long long v, int bytes) {
  for (int b = bytes - 1; b >= 0; --b) out.push_back((unsigned char)(v >> (8 * b)));
}

unsigned long long get_be(const unsigned char *p, int bytes) {
  unsigned long long v = 0;
  for (int b = 0; b < bytes; ++b) v = (v << 8) | p[b];
  return v;
}

int32_t get_i32(const unsigned char *p) { return (int32_t)(uint32_t)get_be(p, 4); }

double get_f64(const unsigned char *p) {
  const unsigned long long u = get_be(p, 8);
  double d;
  std::memcpy(&d, &u, 8);
  return d;
}

void put_f64(std::vector<unsigned char> &out, double d) {
  unsigned long long u;
  std::memcpy(&u, &d, 8);
  put_be(out, u, 8);
}

// read exactly n bytes; 0 on success
PetscErrorCode read_bytes(PetscViewer v, size_t n, std::vector<unsigned char> &buf, const char *what) {
  buf.resize(n);
  const size_t got = n ? std::fread(buf.data(), 1, n, v->f) : 0;
  KSG_CHECK(got == n, PETSC_ERR_FILE_READ, "%s: unexpected end of file while reading %s", v->name.c_str(), what);
  return 0;
}

}  // namespace

extern "C" PetscErrorCode PetscViewerBinaryOpen(MPI_Comm, const char name[], PetscFileMode mode,
                                                PetscViewer *viewer) {
  KSG_CHECK(name && viewer, PETSC_ERR_ARG_NULL, "Null argument");
  KSG_CHECK(mode == FILE_MODE_READ || mode == FILE_MODE_WRITE || mode == FILE_MODE_APPEND, PETSC_ERR_SUP,
            "Unsupported file mode %d", (int)mode);
  const char *fm = mode == FILE_MODE_READ ? "rb" : (mode == FILE_MODE_WRITE ? "wb" : "ab");
  FILE *f = std::fopen(name, fm);
  KSG_CHECK(f, PETSC_ERR_FILE_OPEN, "Cannot open file %s", name);
  PetscViewer v = new _p_PetscViewer();
  v->f = f;
  v->mode = mode;
  v->name = name;
  *viewer = v;
  return 0;
}

extern "C" PetscErrorCode PetscViewerDestroy(PetscViewer *viewer) {
  if (!viewer || !*viewer) return 0;
  PetscViewer v = *viewer;
  const int rc = v->f ? std::fclose(v->f) : 0;
  const std::string name = v->name;
  delete v;
  *viewer = nullptr;
  KSG_CHECK(rc == 0, PETSC_ERR_FILE_WRITE, "Error closing file %s", name.c_str());
  return 0;
}

// An empty sequential AIJ matrix, to be filled by MatLoad (MatCreate + MatSetType(MATSEQAIJ)).
extern "C" PetscErrorCode MatCreate(MPI_Comm, Mat *A) {
  KSG_CHECK(A, PETSC_ERR_ARG_NULL, "Null Mat pointer");
  *A = new _p_Mat();
  (*A)->empty = 1;
  return 0;
}

extern "C" PetscErrorCode MatSetType(Mat A, const char *type) {
  KSG_CHECK(A, PETSC_ERR_ARG_NULL, "Null Mat");
  KSG_CHECK(type && (!std::strcmp(type, "aij") || !std::strcmp(type, "seqaij")), PETSC_ERR_SUP,
            "Only AIJ (CSR) matrices are supported, not '%s'", type ? type : "(null)");
  return 0;
}

extern "C" PetscErrorCode MatSetFromOptions(Mat A) {
  KSG_CHECK(A, PETSC_ERR_ARG_NULL, "Null Mat");
  return 0;
}

extern "C" PetscErrorCode MatGetRowIJ(Mat A, PetscInt shift, PetscBool, PetscBool, PetscInt *n, const PetscInt *ia[],
                                      const PetscInt *ja[], PetscBool *done) {
  KSG_CHECK(A, PETSC_ERR_ARG_NULL, "Null Mat");
  KSG_CHECK(shift == 0, PETSC_ERR_SUP, "Only shift 0 (C indexing) is provided");
  const bool ok = !A->dense && !A->empty;
  if (n) *n = ok ? A->m : 0;
  if (ia) *ia = ok ? A->ai : nullptr;
  if (ja) *ja = ok ? A->aj : nullptr;
  if (done) *done = ok ? PETSC_TRUE : PETSC_FALSE;
  return 0;
}

extern "C" PetscErrorCode MatRestoreRowIJ(Mat A, PetscInt, PetscBool, PetscBool, PetscInt *, const PetscInt *ia[],
                                          const PetscInt *ja[], PetscBool *done) {
  KSG_CHECK(A, PETSC_ERR_ARG_NULL, "Null Mat");
  if (ia) *ia = nullptr;
  if (ja) *ja = nullptr;
  if (done) *done = PETSC_TRUE;
  return 0;
}

extern "C" PetscErrorCode MatSeqAIJGetArrayRead(Mat A, const PetscScalar *array[]) {
  KSG_CHECK(A && array, PETSC_ERR_ARG_NULL, "Null argument");
  KSG_CHECK(!A->dense && !A->empty, PETSC_ERR_ARG_WRONGSTATE, "Not an assembled AIJ matrix");
  *array = A->aa;
  return 0;
}

extern "C" PetscErrorCode MatSeqAIJRestoreArrayRead(Mat A, const PetscScalar *array[]) {
  KSG_CHECK(A, PETSC_ERR_ARG_NULL, "Null Mat");
  if (array) *array = nullptr;
  return 0;
}

// MatLoad_SeqAIJ_Binary: rows, columns, row lengths, column indices, values (PETSc's binary format).
extern "C" PetscErrorCode MatLoad(Mat A, PetscViewer v) {
  KSG_CHECK(A && v, PETSC_ERR_ARG_NULL, "Null argument");
  KSG_CHECK(v->mode == FILE_MODE_READ, PETSC_ERR_ARG_WRONGSTATE, "%s is not open for reading", v->name.c_str());
  KSG_CHECK(A->empty && !A->dense, PETSC_ERR_ARG_WRONGSTATE, "MatLoad needs a Mat from MatCreate that holds no data");
  std::vector<unsigned char> buf;
  KSG_TRY(read_bytes(v, 16, buf, "the matrix header"));
  const int32_t classid = get_i32(&buf[0]), m = get_i32(&buf[4]), n = get_i32(&buf[8]), nz = get_i32(&buf[12]);
  KSG_CHECK(classid == MAT_FILE_CLASSID, PETSC_ERR_FILE_UNEXPECTED, "%s: not a matrix (class id %d)",
            v->name.c_str(), classid);
  KSG_CHECK(m >= 0 && n >= 0, PETSC_ERR_FILE_UNEXPECTED, "%s: negative dimensions", v->name.c_str());
  KSG_CHECK(nz >= 0, PETSC_ERR_FILE_UNEXPECTED,
            "%s: matrix stored in a special format on disk (nonzeros %d), cannot load as AIJ", v->name.c_str(), nz);
  KSG_TRY(read_bytes(v, 4 * (size_t)m, buf, "the row lengths"));
  std::vector<PetscInt> ai(m + 1);
  ai[0] = 0;
  long long total = 0;
  for (int r = 0; r < m; ++r) {
    const int32_t len = get_i32(&buf[4 * (size_t)r]);
    KSG_CHECK(len >= 0 && len <= n, PETSC_ERR_FILE_UNEXPECTED, "%s: row %d has length %d", v->name.c_str(), r, len);
    total += len;
    KSG_CHECK(total <= nz, PETSC_ERR_FILE_UNEXPECTED, "%s: row lengths exceed the nonzero count", v->name.c_str());
    ai[r + 1] = (PetscInt)total;
  }
  KSG_CHECK(total == nz, PETSC_ERR_FILE_UNEXPECTED, "%s: row lengths sum to %lld, header says %d", v->name.c_str(),
            total, nz);
  KSG_TRY(read_bytes(v, 4 * (size_t)nz, buf, "the column indices"));
  std::vector<PetscInt> aj(nz);
  for (size_t p = 0; p < (size_t)nz; ++p) aj[p] = get_i32(&buf[4 * p]);
  KSG_TRY(read_bytes(v, 8 * (size_t)nz, buf, "the values"));
  std::vector<double> aa(nz);
  for (size_t p = 0; p < (size_t)nz; ++p) aa[p] = get_f64(&buf[8 * p]);
  for (int r = 0; r < m; ++r)
    for (int p = ai[r]; p < ai[r + 1]; ++p) {
      KSG_CHECK(aj[p] >= 0 && aj[p] < n, PETSC_ERR_FILE_UNEXPECTED, "%s: column index %d out of range in row %d",
                v->name.c_str(), aj[p], r);
      KSG_CHECK(std::isfinite(aa[p]), PETSC_ERR_FILE_UNEXPECTED, "%s: entry (%d,%d) is not finite",
                v->name.c_str(), r, aj[p]);
    }
  A->own_i.swap(ai);
  A->own_j.swap(aj);
  A->own_a.swap(aa);
  A->m = m;
  A->n = n;
  A->ai = A->own_i.data();
  A->aj = A->own_j.data();
  A->aa = A->own_a.data();
  A->nnz = nz;
  A->empty = 0;
  return 0;
}

// MatView with a binary viewer: the same layout MatLoad reads
extern "C" PetscErrorCode MatView(Mat A, PetscViewer v) {
  KSG_CHECK(A && v, PETSC_ERR_ARG_NULL, "Null argument");
  KSG_CHECK(v->mode != FILE_MODE_READ, PETSC_ERR_ARG_WRONGSTATE, "%s is not open for writing", v->name.c_str());
  KSG_CHECK(!A->dense && !A->empty, PETSC_ERR_SUP, "MatView writes AIJ matrices only");
  std::vector<unsigned char> out;
  out.reserve(16 + 4 * (size_t)A->m + 12 * (size_t)A->nnz);
  put_be(out, (uint32_t)MAT_FILE_CLASSID, 4);
  put_be(out, (uint32_t)A->m, 4);
  put_be(out, (uint32_t)A->n, 4);
  put_be(out, (uint32_t)A->nnz, 4);
  for (int r = 0; r < A->m; ++r) put_be(out, (uint32_t)(A->ai[r + 1] - A->ai[r]), 4);
  for (long long p = 0; p < A->nnz; ++p) put_be(out, (uint32_t)A->aj[p], 4);
  for (long long p = 0; p < A->nnz; ++p) put_f64(out, A->aa[p]);
  KSG_CHECK(std::fwrite(out.data(), 1, out.size(), v->f) == out.size(), PETSC_ERR_FILE_WRITE,
            "%s: write failed", v->name.c_str());
  return 0;
}

extern "C" PetscErrorCode VecLoad(Vec x, PetscViewer v) {
  KSG_CHECK(x && v, PETSC_ERR_ARG_NULL, "Null argument");
  KSG_CHECK(v->mode == FILE_MODE_READ, PETSC_ERR_ARG_WRONGSTATE, "%s is not open for reading", v->name.c_str());
  std::vector<unsigned char> buf;
  KSG_TRY(read_bytes(v, 8, buf, "the vector header"));
  const int32_t classid = get_i32(&buf[0]), n = get_i32(&buf[4]);
  KSG_CHECK(classid == VEC_FILE_CLASSID, PETSC_ERR_FILE_UNEXPECTED, "%s: not a vector (class id %d)",
            v->name.c_str(), classid);
  KSG_CHECK(n >= 0, PETSC_ERR_FILE_UNEXPECTED, "%s: negative vector length", v->name.c_str());
  KSG_CHECK(x->n == 0 || x->n == n, PETSC_ERR_ARG_SIZ, "%s: vector of length %d, the Vec has %d", v->name.c_str(),
            n, x->n);
  KSG_TRY(read_bytes(v, 8 * (size_t)n, buf, "the vector values"));
  if (x->n == 0) {
    x->own.assign(n, 0.0);
    x->a = x->own.data();
    x->n = n;
  }
  for (int i = 0; i < n; ++i) x->a[i] = get_f64(&buf[8 * (size_t)i]);
  return 0;
}

extern "C" PetscErrorCode VecView(Vec x, PetscViewer v) {
  KSG_CHECK(x && v, PETSC_ERR_ARG_NULL, "Null argument");
  KSG_CHECK(v->mode != FILE_MODE_READ, PETSC_ERR_ARG_WRONGSTATE, "%s is not open for writing", v->name.c_str());
  std::vector<unsigned char> out;
  put_be(out, (uint32_t)VEC_FILE_CLASSID, 4);
  put_be(out, (uint32_t)x->n, 4);
  for (int i = 0; i < x->n; ++i) put_f64(out, x->a[i]);
  KSG_CHECK(std::fwrite(out.data(), 1, out.size(), v->f) == out.size(), PETSC_ERR_FILE_WRITE,
            "%s: write failed", v->name.c_str());
  return 0;
}
