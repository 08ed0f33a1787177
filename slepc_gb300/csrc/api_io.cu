// api_io.cu -- viewers: PETSc binary matrix and vector files (PetscViewerBinaryOpen, MatLoad, MatView, VecLoad,
// VecView) and the ASCII result reports of EPS (EPSErrorView, EPSConvergedReasonView, EPSValuesView).
//
// The reference's tutorials read their operators this way (src/eps/tutorials/ex4.c:45-49, ex7.c:52, ex31.c:551-562),
// and its data files (share/slepc/datafiles/matrices/*.petsc) use PETSc's binary format: every item big-endian,
//   matrix: int32 MAT_FILE_CLASSID, rows, columns, nonzeros; int32 row lengths[rows]; int32 column indices[nnz];
//           float64 values[nnz];
//   vector: int32 VEC_FILE_CLASSID, length; float64 values[length].
// Items are assembled byte by byte, so the files read and write the same on little- and big-endian hosts.  A loaded
// matrix owns its CSR arrays; everything else about it (device upload on first solve, MatMult, MatDestroy) is the
// same as for MatCreateSeqAIJWithArrays.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "internal.h"


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
  if (v->borrowed) {
    *viewer = nullptr;
    return 0;
  }
  const int rc = (v->f && v->f != stdout && v->f != stderr) ? std::fclose(v->f) : 0;
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
  KSG_CHECK(!v->ascii, PETSC_ERR_SUP, "Only binary viewers are supported here");
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
  A->state++;
  return 0;
}

namespace {
PetscErrorCode mat_view_ascii(Mat A, PetscViewer v);
}

// MatView: a binary viewer writes the layout MatLoad reads; an ASCII viewer (NULL is PETSC_VIEWER_STDOUT_WORLD)
// prints the rows as PETSc's seqaij viewer does
extern "C" PetscErrorCode MatView(Mat A, PetscViewer v) {
  KSG_CHECK(A, PETSC_ERR_ARG_NULL, "Null argument");
  KSG_CHECK(A->pending.empty() && !A->empty, PETSC_ERR_ARG_WRONGSTATE, "Not for unassembled matrix");
  if (!v || v->ascii) return mat_view_ascii(A, v);
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
  KSG_CHECK(!v->ascii, PETSC_ERR_SUP, "Only binary viewers are supported here");
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
  KSG_CHECK(!v->ascii, PETSC_ERR_SUP, "Only binary viewers are supported here");
  KSG_CHECK(v->mode != FILE_MODE_READ, PETSC_ERR_ARG_WRONGSTATE, "%s is not open for writing", v->name.c_str());
  std::vector<unsigned char> out;
  put_be(out, (uint32_t)VEC_FILE_CLASSID, 4);
  put_be(out, (uint32_t)x->n, 4);
  for (int i = 0; i < x->n; ++i) put_f64(out, x->a[i]);
  KSG_CHECK(std::fwrite(out.data(), 1, out.size(), v->f) == out.size(), PETSC_ERR_FILE_WRITE,
            "%s: write failed", v->name.c_str());
  return 0;
}

// ---------------------------------------------------------------------------------------------------------------
// ASCII viewers (PetscViewerASCIIOpen, PetscViewerASCIIGetStdout, PETSC_VIEWER_STDOUT_WORLD/SELF) with a format
// stack, and the EPS result reports the reference's tutorials print (src/eps/interface/epsview.c)
// ---------------------------------------------------------------------------------------------------------------
namespace {

_p_PetscViewer *stdout_viewer() {
  static _p_PetscViewer v = [] {
    _p_PetscViewer w;
    w.f = stdout;
    w.mode = FILE_MODE_WRITE;
    w.name = "stdout";
    w.ascii = 1;
    w.borrowed = 1;
    return w;
  }();
  return &v;
}

PetscViewerFormat top_format(PetscViewer v) { return v->formats.empty() ? PETSC_VIEWER_DEFAULT : v->formats.back(); }

struct Text {
  std::string s;
  void add(const char *fmt, ...) {
    char buf[256];
    va_list ap;
    va_start(ap, fmt);
    const int n = std::vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    if (n > 0) s.append(buf, std::min<size_t>((size_t)n, sizeof(buf) - 1));
  }
  // one eigenvalue as SlepcPrintEigenvalueASCII prints it (include/slepc/private/slepcimpl.h:92-112): five decimals,
  // a part below 1e-10 (PETSC_SMALL) of the other printed as zero, real when the imaginary part is zero
  void eig(double re, double im) {
    const double small = 1e-10;
    if (im != 0.0 && std::fabs(re) / std::fabs(im) < small) re = 0.0;
    if (re != 0.0 && std::fabs(im) / std::fabs(re) < small) im = 0.0;
    if (im != 0.0) add("%.5f%+.5fi", re, im);
    else add("%.5f", re);
  }
};

PetscErrorCode emit(PetscViewer v, const Text &t) {
  if (t.s.empty()) return 0;
  KSG_CHECK(std::fwrite(t.s.data(), 1, t.s.size(), v->f) == t.s.size(), PETSC_ERR_FILE_WRITE, "%s: write failed",
            v->name.c_str());
  std::fflush(v->f);
  return 0;
}

// the name MATLAB-format reports print: the one given by PetscObjectSetName, else "eps"
const char *eps_name(EPS eps) { return eps->name.empty() ? "eps" : eps->name.c_str(); }

// %g as PETSc's ASCII viewers print it: a value that prints as an integer gets a trailing decimal point ("20.")
void add_g(Text &t, double x) {
  char buf[64];
  std::snprintf(buf, sizeof(buf), "%g", x);
  if (!std::strpbrk(buf, ".eEni")) std::strncat(buf, ".", sizeof(buf) - std::strlen(buf) - 1);
  t.s += buf;
}

// MatView_SeqAIJ_ASCII / MatView_SeqDense_ASCII in the default format: the object header, then one line per row,
// " (column, value) " for each stored entry of an AIJ matrix, every value of a dense one
PetscErrorCode mat_view_ascii(Mat A, PetscViewer v) {
  if (!v) v = stdout_viewer();
  Text t;
  t.add("Mat Object: 1 MPI process\n  type: %s\n", A->dense ? "seqdense" : "seqaij");
  const PetscViewerFormat fmt = top_format(v);
  if (fmt == PETSC_VIEWER_ASCII_INFO || fmt == PETSC_VIEWER_ASCII_INFO_DETAIL) {
    const long long nz = A->dense ? (long long)A->m * A->n : A->nnz;
    t.add("  rows=%d, cols=%d\n  total: nonzeros=%lld, allocated nonzeros=%lld\n", A->m, A->n, nz, nz);
    return emit(v, t);
  }
  for (int r = 0; r < A->m; ++r) {
    if (A->dense) {
      for (int c = 0; c < A->n; ++c) t.add("%18.16e ", A->data[(size_t)c * A->lda + r]);
    } else {
      t.add("row %d:", r);
      for (PetscInt p = A->ai[r]; p < A->ai[r + 1]; ++p) {
        t.add(" (%d, ", (int)A->aj[p]);
        add_g(t, A->aa[p]);
        t.s += ") ";
      }
    }
    t.s += "\n";
  }
  return emit(v, t);
}

const char *reason_name(int reason) {
  switch (reason) {
    case EPS_CONVERGED_TOL: return "CONVERGED_TOL";
    case EPS_CONVERGED_USER: return "CONVERGED_USER";
    case EPS_DIVERGED_ITS: return "DIVERGED_ITS";
    case EPS_DIVERGED_BREAKDOWN: return "DIVERGED_BREAKDOWN";
    case EPS_DIVERGED_SYMMETRY_LOST: return "DIVERGED_SYMMETRY_LOST";
    default: return "CONVERGED_ITERATING";
  }
}

}  // namespace

extern "C" PetscViewer PETSC_VIEWER_STDOUT_(MPI_Comm) { return stdout_viewer(); }

extern "C" PetscErrorCode PetscViewerASCIIGetStdout(MPI_Comm, PetscViewer *viewer) {
  KSG_CHECK(viewer, PETSC_ERR_ARG_NULL, "Null argument");
  *viewer = stdout_viewer();
  return 0;
}

// PetscViewerASCIIOpen: a text file written from the start; the names "stdout" and "stderr" give those streams
extern "C" PetscErrorCode PetscViewerASCIIOpen(MPI_Comm, const char name[], PetscViewer *viewer) {
  KSG_CHECK(name && viewer, PETSC_ERR_ARG_NULL, "Null argument");
  FILE *f = !std::strcmp(name, "stdout") ? stdout : !std::strcmp(name, "stderr") ? stderr : std::fopen(name, "w");
  KSG_CHECK(f, PETSC_ERR_FILE_OPEN, "Cannot open file %s", name);
  PetscViewer v = new _p_PetscViewer();
  v->f = f;
  v->mode = FILE_MODE_WRITE;
  v->name = name;
  v->ascii = 1;
  *viewer = v;
  return 0;
}

extern "C" PetscErrorCode PetscViewerPushFormat(PetscViewer v, PetscViewerFormat format) {
  KSG_CHECK(v, PETSC_ERR_ARG_NULL, "Null viewer");
  KSG_CHECK(v->formats.size() < 10, PETSC_ERR_ARG_OUTOFRANGE, "Too many PetscViewerPushFormat() calls");
  v->formats.push_back(format);
  return 0;
}

extern "C" PetscErrorCode PetscViewerPopFormat(PetscViewer v) {
  KSG_CHECK(v, PETSC_ERR_ARG_NULL, "Null viewer");
  if (!v->formats.empty()) v->formats.pop_back();
  return 0;
}

extern "C" PetscErrorCode PetscViewerGetFormat(PetscViewer v, PetscViewerFormat *format) {
  KSG_CHECK(v && format, PETSC_ERR_ARG_NULL, "Null argument");
  *format = top_format(v);
  return 0;
}

extern "C" PetscErrorCode PetscViewerASCIIPrintf(PetscViewer v, const char format[], ...) {
  KSG_CHECK(v && format, PETSC_ERR_ARG_NULL, "Null argument");
  KSG_CHECK(v->ascii, PETSC_ERR_ARG_WRONG, "%s is not an ASCII viewer", v->name.c_str());
  va_list ap;
  va_start(ap, format);
  const int rc = std::vfprintf(v->f, format, ap);
  va_end(ap);
  KSG_CHECK(rc >= 0, PETSC_ERR_FILE_WRITE, "%s: write failed", v->name.c_str());
  std::fflush(v->f);
  return 0;
}

// EPSConvergedReasonView (epsview.c:243-262): one line with the number of converged pairs, the reason and the
// number of restarts; PETSC_VIEWER_FAILED prints only a failure
extern "C" PetscErrorCode EPSConvergedReasonView(EPS eps, PetscViewer v) {
  KSG_CHECK(eps, PETSC_ERR_ARG_NULL, "Null EPS");
  if (!v) v = stdout_viewer();
  if (!v->ascii) return 0;
  const int nconv = eps->nconv, its = eps->its, reason = eps->reason;  // before EPSSolve: 0, CONVERGED_ITERATING
  Text t;
  if (reason > 0 && top_format(v) != PETSC_VIEWER_FAILED)
    t.add("%s Linear eigensolve converged (%d eigenpair%s) due to %s; iterations %d\n", eps->prefix.c_str(), nconv,
          nconv > 1 ? "s" : "", reason_name(reason), its);
  else if (reason <= 0)
    t.add("%s Linear eigensolve did not converge due to %s; iterations %d\n", eps->prefix.c_str(), reason_name(reason),
          its);
  return emit(v, t);
}

// EPSErrorView (epsview.c:297-447).  Default / ASCII_INFO format: the first nev eigenvalues, eight to a line, when
// all of them converged with errors below 5*tol, else a one-line diagnosis.  ASCII_INFO_DETAIL: a table of every
// converged eigenvalue with its error.  Other formats print nothing.
extern "C" PetscErrorCode EPSErrorView(EPS eps, EPSErrorType etype, PetscViewer v) {
  KSG_CHECK(eps, PETSC_ERR_ARG_NULL, "Null EPS");
  KSG_CHECK(eps->solved, PETSC_ERR_ORDER, "Must call EPSSolve() first");
  if (!v) v = stdout_viewer();
  if (!v->ascii) return 0;
  PetscInt nconv = 0, nev = 0;
  PetscReal tol = 0.0;
  KSG_TRY(EPSGetConverged(eps, &nconv));
  KSG_TRY(EPSGetDimensions(eps, &nev, nullptr, nullptr));
  KSG_TRY(EPSGetTolerances(eps, &tol, nullptr));
  const PetscViewerFormat fmt = top_format(v);
  Text t;
  if (fmt == PETSC_VIEWER_DEFAULT || fmt == PETSC_VIEWER_ASCII_INFO) {
    if (nconv < nev) {
      t.add(" Problem: less than %d eigenvalues converged\n\n", (int)nev);
      return emit(v, t);
    }
    for (PetscInt i = 0; i < nev; ++i) {
      PetscReal err = 0.0;
      KSG_TRY(EPSComputeError(eps, i, etype, &err));
      if (err >= 5.0 * tol) {
        t.add(" Problem: some of the first %d relative errors are higher than the tolerance\n\n", (int)nev);
        return emit(v, t);
      }
    }
    t.add(" All requested eigenvalues computed up to the required tolerance:");
    for (PetscInt i = 0; i < nev; ++i) {
      if (i % 8 == 0) t.add("\n     ");
      PetscScalar kr = 0.0, ki = 0.0;
      KSG_TRY(EPSGetEigenvalue(eps, i, &kr, &ki));
      t.eig(kr, ki);
      if (i + 1 < nev) t.add(", ");
    }
    t.add("\n\n");
  } else if (fmt == PETSC_VIEWER_ASCII_INFO_DETAIL) {
    if (!nconv) return 0;
    const char *sep = " ---------------------- --------------------\n";
    const bool gen = eps->B != nullptr;
    const char *head = etype == EPS_ERROR_ABSOLUTE   ? (gen ? "   ||Ax-kBx||" : "   ||Ax-kx||")
                       : etype == EPS_ERROR_RELATIVE ? (gen ? "||Ax-kBx||/||kx||" : "||Ax-kx||/||kx||")
                                                     : "    eta(x,k)";
    t.add("%s            k             %s\n%s", sep, head, sep);
    for (PetscInt i = 0; i < nconv; ++i) {
      PetscScalar kr = 0.0, ki = 0.0;
      PetscReal err = 0.0;
      KSG_TRY(EPSGetEigenvalue(eps, i, &kr, &ki));
      KSG_TRY(EPSComputeError(eps, i, etype, &err));
      if (ki != 0.0) t.add("  % 9f%+9fi      %12g\n", kr, ki, err);
      else t.add("    % 12f           %12g\n", kr, err);
    }
    t.add("%s", sep);
  } else if (fmt == PETSC_VIEWER_ASCII_MATLAB) {
    // EPSErrorView_MATLAB (epsview.c:372-388)
    t.add("Error_%s = [\n", eps_name(eps));
    for (PetscInt i = 0; i < nconv; ++i) {
      PetscReal err = 0.0;
      KSG_TRY(EPSComputeError(eps, i, etype, &err));
      t.add("%18.16e\n", err);
    }
    t.add("];\n");
  }
  return emit(v, t);
}

// EPSValuesView (epsview.c:603-617), ASCII: every converged eigenvalue on its own line
extern "C" PetscErrorCode EPSValuesView(EPS eps, PetscViewer v) {
  KSG_CHECK(eps, PETSC_ERR_ARG_NULL, "Null EPS");
  KSG_CHECK(eps->solved, PETSC_ERR_ORDER, "Must call EPSSolve() first");
  if (!v) v = stdout_viewer();
  if (!v->ascii) return 0;
  PetscInt nconv = 0;
  KSG_TRY(EPSGetConverged(eps, &nconv));
  Text t;
  if (top_format(v) == PETSC_VIEWER_ASCII_MATLAB) {
    // EPSValuesView_MATLAB (epsview.c:619-646)
    t.add("Lambda_%s = [\n", eps_name(eps));
    for (PetscInt i = 0; i < nconv; ++i) {
      PetscScalar kr = 0.0, ki = 0.0;
      KSG_TRY(EPSGetEigenvalue(eps, i, &kr, &ki));
      if (ki != 0.0) t.add("%18.16e%+18.16ei\n", kr, ki);
      else t.add("%18.16e\n", kr);
    }
    t.add("];\n");
    return emit(v, t);
  }
  t.add("Eigenvalues = \n");
  for (PetscInt i = 0; i < nconv; ++i) {
    PetscScalar kr = 0.0, ki = 0.0;
    KSG_TRY(EPSGetEigenvalue(eps, i, &kr, &ki));
    t.add("   ");
    t.eig(kr, ki);
    t.add("\n");
  }
  t.add("\n");
  return emit(v, t);
}

// ---------------------------------------------------------------------------------------------------------------
// object names, viewer-and-format pairs, and the EPS monitors of epsmon.c
// ---------------------------------------------------------------------------------------------------------------
extern "C" PetscErrorCode PetscObjectSetName(PetscObject obj, const char name[]) {
  KSG_CHECK(obj && name, PETSC_ERR_ARG_NULL, "Null argument");
  if (*static_cast<const unsigned *>(obj) == KSG_EPS_COOKIE) static_cast<EPS>(obj)->name = name;
  return 0;  // names of other objects are not printed anywhere
}

extern "C" PetscErrorCode PetscObjectGetName(PetscObject obj, const char *name[]) {
  KSG_CHECK(obj && name, PETSC_ERR_ARG_NULL, "Null argument");
  *name = (*static_cast<const unsigned *>(obj) == KSG_EPS_COOKIE) ? eps_name(static_cast<EPS>(obj)) : "";
  return 0;
}

namespace {
// every PetscViewerAndFormat is allocated with this tail: whether it owns its viewer (options-created file viewers)
struct VfBox {
  PetscViewerAndFormat vf;
  int owns_viewer;
  PetscInt oldnconv;  // EPSMonitorConverged
};
}  // namespace

extern "C" PetscErrorCode PetscViewerAndFormatCreate(PetscViewer viewer, PetscViewerFormat format,
                                                     PetscViewerAndFormat **vf) {
  KSG_CHECK(vf, PETSC_ERR_ARG_NULL, "Null argument");
  VfBox *b = new VfBox();
  b->vf.viewer = viewer ? viewer : stdout_viewer();
  b->vf.format = format;
  b->vf.data = nullptr;
  *vf = &b->vf;
  return 0;
}

extern "C" PetscErrorCode PetscViewerAndFormatDestroy(PetscViewerAndFormat **vf) {
  if (!vf || !*vf) return 0;
  VfBox *b = reinterpret_cast<VfBox *>(*vf);
  if (b->owns_viewer) KSG_TRY(PetscViewerDestroy(&b->vf.viewer));
  delete b;
  *vf = nullptr;
  return 0;
}

extern "C" PetscErrorCode EPSMonitorConvergedCreate(PetscViewer viewer, PetscViewerFormat format, void *,
                                                    PetscViewerAndFormat **vf) {
  KSG_TRY(PetscViewerAndFormatCreate(viewer, format, vf));
  reinterpret_cast<VfBox *>(*vf)->vf.data = &reinterpret_cast<VfBox *>(*vf)->oldnconv;
  return 0;
}

extern "C" PetscErrorCode EPSMonitorConvergedDestroy(PetscViewerAndFormat **vf) {
  return PetscViewerAndFormatDestroy(vf);
}

namespace {
// one monitor line's eigenvalue: " %g", then "%+gi" for a nonzero imaginary part (epsmon.c:205-212)
void add_monitor_value(Text &t, double er, double ei) {
  t.s += ' ';
  add_g(t, er);
  if (ei != 0.0) {
    char buf[64];
    std::snprintf(buf, sizeof(buf), "%+g", ei);
    t.s += buf;
    if (!std::strpbrk(buf + 1, ".eEni")) t.s += '.';
    t.s += 'i';
  }
}

PetscErrorCode monitor_viewer(EPS eps, PetscViewerAndFormat *vf, PetscViewer *v) {
  KSG_CHECK(eps && vf, PETSC_ERR_ARG_NULL, "Null argument");
  *v = vf->viewer ? vf->viewer : stdout_viewer();
  return 0;
}
}  // namespace

// EPSMonitorFirst (epsmon.c:183-220): the first unconverged value and its error estimate
extern "C" PetscErrorCode EPSMonitorFirst(EPS eps, PetscInt its, PetscInt nconv, PetscScalar eigr[],
                                          PetscScalar eigi[], PetscReal errest[], PetscInt nest,
                                          PetscViewerAndFormat *vf) {
  PetscViewer v;
  KSG_TRY(monitor_viewer(eps, vf, &v));
  if (!v->ascii) return 0;
  Text t;
  if (its == 1 && !eps->prefix.empty())
    t.add("  Eigenvalue approximations and residual norms for %s solve.\n", eps->prefix.c_str());
  if (nconv >= nest) return emit(v, t);
  t.add("%3d EPS nconv=%d first unconverged value (error)", (int)its, (int)nconv);
  add_monitor_value(t, eigr[nconv], eigi[nconv]);
  t.add(" (%10.8e)\n", errest[nconv]);
  return emit(v, t);
}

// EPSMonitorAll (epsmon.c:236-270): every current value and error estimate
extern "C" PetscErrorCode EPSMonitorAll(EPS eps, PetscInt its, PetscInt nconv, PetscScalar eigr[], PetscScalar eigi[],
                                        PetscReal errest[], PetscInt nest, PetscViewerAndFormat *vf) {
  PetscViewer v;
  KSG_TRY(monitor_viewer(eps, vf, &v));
  if (!v->ascii) return 0;
  Text t;
  if (its == 1 && !eps->prefix.empty())
    t.add("  Eigenvalue approximations and residual norms for %s solve.\n", eps->prefix.c_str());
  t.add("%3d EPS nconv=%d Values (Errors)", (int)its, (int)nconv);
  for (PetscInt i = 0; i < nest; ++i) {
    add_monitor_value(t, eigr[i], eigi[i]);
    t.add(" (%10.8e)", errest[i]);
  }
  t.add("\n");
  return emit(v, t);
}

// EPSMonitorConverged (epsmon.c:291-330): each value once, in the restart where it converged
extern "C" PetscErrorCode EPSMonitorConverged(EPS eps, PetscInt its, PetscInt nconv, PetscScalar eigr[],
                                              PetscScalar eigi[], PetscReal errest[], PetscInt,
                                              PetscViewerAndFormat *vf) {
  PetscViewer v;
  KSG_TRY(monitor_viewer(eps, vf, &v));
  KSG_CHECK(vf->data, PETSC_ERR_ARG_WRONG, "EPSMonitorConverged needs the context of EPSMonitorConvergedCreate");
  PetscInt *old = static_cast<PetscInt *>(vf->data);
  if (!v->ascii) return 0;
  Text t;
  if (its == 1 && !eps->prefix.empty()) t.add("  Convergence history for %s solve.\n", eps->prefix.c_str());
  if (its == 1) *old = 0;
  if (*old == nconv) return emit(v, t);
  for (PetscInt i = *old; i < nconv; ++i) {
    t.add("%3d EPS converged value (error) #%d", (int)its, (int)i);
    add_monitor_value(t, eigr[i], eigi[i]);
    t.add(" (%10.8e)\n", errest[i]);
  }
  *old = nconv;
  return emit(v, t);
}

// A viewer from an options value "[ascii][:file][:format]" (PetscOptionsCreateViewer): stdout unless a file is
// named (opened for appending, owned by the caller); the draw and binary viewer types are not provided (*ok = 0)
PetscErrorCode ksg_viewer_from_spec(const char *spec, PetscViewer *viewer, PetscViewerFormat *format, int *ok) {
  *viewer = stdout_viewer();
  *format = PETSC_VIEWER_DEFAULT;
  *ok = 1;
  if (!spec || !*spec) return 0;
  std::string sp(spec), type, file, fmt;
  const size_t c1 = sp.find(':');
  type = sp.substr(0, c1);
  if (c1 != std::string::npos) {
    const size_t c2 = sp.find(':', c1 + 1);
    file = sp.substr(c1 + 1, c2 == std::string::npos ? std::string::npos : c2 - c1 - 1);
    if (c2 != std::string::npos) fmt = sp.substr(c2 + 1);
  }
  if (!type.empty() && type != "ascii") {
    *ok = 0;
    return 0;
  }
  if (fmt == "ascii_info") *format = PETSC_VIEWER_ASCII_INFO;
  else if (fmt == "ascii_info_detail") *format = PETSC_VIEWER_ASCII_INFO_DETAIL;
  else if (fmt == "ascii_matlab") *format = PETSC_VIEWER_ASCII_MATLAB;
  else if (fmt == "failed") *format = PETSC_VIEWER_FAILED;
  else KSG_CHECK(fmt.empty() || fmt == "default", PETSC_ERR_SUP, "Unsupported viewer format %s", fmt.c_str());
  if (!file.empty() && file != "stdout") {
    FILE *f = file == "stderr" ? stderr : std::fopen(file.c_str(), "a");
    KSG_CHECK(f, PETSC_ERR_FILE_OPEN, "Cannot open file %s", file.c_str());
    PetscViewer v = new _p_PetscViewer();
    v->f = f;
    v->mode = FILE_MODE_APPEND;
    v->name = file;
    v->ascii = 1;
    *viewer = v;
  }
  return 0;
}

// a monitor from the options database (-eps_monitor[_all|_conv] [spec]): kind 0 first, 1 all, 2 converged
PetscErrorCode ksg_eps_monitor_from_spec(EPS eps, int kind, const char *spec) {
  PetscViewer v;
  PetscViewerFormat f;
  int ok;
  KSG_TRY(ksg_viewer_from_spec(spec, &v, &f, &ok));
  if (!ok) return 0;  // draw and binary monitors are not provided: nothing is printed
  PetscViewerAndFormat *vf;
  if (kind == 2) KSG_TRY(EPSMonitorConvergedCreate(v, f, nullptr, &vf));
  else KSG_TRY(PetscViewerAndFormatCreate(v, f, &vf));
  reinterpret_cast<VfBox *>(vf)->owns_viewer = !v->borrowed;
  EPSMonitorFn *fn = kind == 0   ? reinterpret_cast<EPSMonitorFn *>(EPSMonitorFirst)
                     : kind == 1 ? reinterpret_cast<EPSMonitorFn *>(EPSMonitorAll)
                                 : reinterpret_cast<EPSMonitorFn *>(EPSMonitorConverged);
  PetscErrorCode ierr = EPSMonitorSet(eps, fn, vf, reinterpret_cast<PetscCtxDestroyFn *>(PetscViewerAndFormatDestroy));
  if (ierr) PetscViewerAndFormatDestroy(&vf);
  return ierr;
}

// the reports EPSSolve prints when it ends, in the order of epssolve.c:182-186: view, converged reason, errors,
// values
PetscErrorCode ksg_eps_post_views(EPS eps) {
  std::vector<EPSPostView> views = eps->post_views;
  std::stable_sort(views.begin(), views.end(), [](const EPSPostView &a, const EPSPostView &b) {
    return (a.kind + 1) % 4 < (b.kind + 1) % 4;  // view (3), converged reason (0), errors (1), values (2)
  });
  for (const EPSPostView &pv : views) {
    PetscViewer v;
    PetscViewerFormat f;
    int ok;
    std::string spec = pv.file.empty() ? std::string() : "ascii:" + pv.file;
    KSG_TRY(ksg_viewer_from_spec(spec.c_str(), &v, &f, &ok));
    v->formats.push_back(pv.format);
    PetscErrorCode ierr = pv.kind == 0   ? EPSConvergedReasonView(eps, v)
                          : pv.kind == 1 ? EPSErrorView(eps, (EPSErrorType)pv.etype, v)
                          : pv.kind == 2 ? EPSValuesView(eps, v)
                                         : EPSView(eps, v);
    v->formats.pop_back();
    if (!v->borrowed) PetscViewerDestroy(&v);
    KSG_TRY(ierr);
  }
  return 0;
}

// EPSView (epsview.c:40-190 with EPSView_KrylovSchur, krylovschur.c:1490-1500): the solver configuration, then the
// basis, projected-problem and spectral-transformation objects.  Before EPSSetUp the values are the ones set;
// after it, the ones in use.  The BV lines state this library's basis (device, pair or FP64 storage, two-pass
// delayed classical Gram-Schmidt) rather than the reference's default settings.
extern "C" PetscErrorCode EPSView(EPS eps, PetscViewer v) {
  KSG_CHECK(eps, PETSC_ERR_ARG_NULL, "Null EPS");
  if (!v) v = stdout_viewer();
  if (!v->ascii) return 0;
  Text t;
  t.add("EPS Object: %s%s1 MPI process\n", eps->name.c_str(), eps->name.empty() ? "" : " ");
  t.add("  type: krylovschur\n");
  t.add("    %d%% of basis vectors kept after restart\n", (int)(100 * eps->keep));
  t.add("    using the %slocking variant\n", eps->lock ? "" : "non-");
  const char *ptype = "not yet set";
  switch (eps->problem) {
    case EPS_HEP: ptype = "symmetric eigenvalue problem"; break;
    case EPS_GHEP: ptype = "generalized symmetric eigenvalue problem"; break;
    case EPS_NHEP: ptype = "non-symmetric eigenvalue problem"; break;
    case EPS_GNHEP: ptype = "generalized non-symmetric eigenvalue problem"; break;
    default: break;
  }
  t.add("  problem type: %s\n", ptype);
  if (eps->extraction == EPS_HARMONIC) t.add("  extraction type: harmonic Ritz\n");
  t.add("  selected portion of the spectrum: ");
  char tg[64];
  std::snprintf(tg, sizeof(tg), "%g", eps->target);
  if (!std::strpbrk(tg, ".eEni")) std::strncat(tg, ".", sizeof(tg) - std::strlen(tg) - 1);
  switch (eps->which) {
    case EPS_TARGET_MAGNITUDE: t.add("closest to target: %s (in magnitude)\n", tg); break;
    case EPS_TARGET_REAL: t.add("closest to target: %s (along the real axis)\n", tg); break;
    case EPS_LARGEST_MAGNITUDE: t.add("largest eigenvalues in magnitude\n"); break;
    case EPS_SMALLEST_MAGNITUDE: t.add("smallest eigenvalues in magnitude\n"); break;
    case EPS_LARGEST_REAL: t.add("largest real parts\n"); break;
    case EPS_SMALLEST_REAL: t.add("smallest real parts\n"); break;
    case EPS_LARGEST_IMAGINARY: t.add("largest imaginary parts\n"); break;
    case EPS_SMALLEST_IMAGINARY: t.add("smallest imaginary parts\n"); break;
    default: t.add("not yet set\n"); break;
  }
  // purification applies to definite generalised problems only (epssetup.c:359-368)
  const bool purify = eps->purify && (!eps->setup || (eps->B && eps->problem == EPS_GHEP));
  if (purify) t.add("  postprocessing eigenvectors with purification\n");
  t.add("  number of eigenvalues (nev): %d\n", eps->setup ? eps->nev_e : eps->nev);
  t.add("  number of column vectors (ncv): %d\n", eps->setup ? eps->ncv_e : eps->ncv);
  t.add("  maximum dimension of projected problem (mpd): %d\n", eps->setup ? eps->mpd_e : eps->mpd);
  t.add("  maximum number of iterations: %d\n", eps->setup ? eps->maxit_e : eps->max_it);
  t.add("  tolerance: %g\n", eps->setup ? eps->tol_e : eps->tol);
  t.add("  convergence test: ");
  if (eps->conv == EPS_CONV_ABS) t.add("absolute\n");
  else if (eps->conv == EPS_CONV_NORM) {
    t.add("relative to the eigenvalue and matrix norms\n");
    t.add("  computed matrix norms: norm(A)=%g", eps->nrma);
    if (eps->B) t.add(", norm(B)=%g", eps->nrmb);
    t.add("\n");
  } else t.add("relative to the eigenvalue\n");
  if (!eps->v0.empty()) t.add("  dimension of user-provided initial space: 1\n");
  const int ncv = eps->setup ? eps->ncv_e : eps->ncv;
  t.add("BV Object: 1 MPI process\n");
  t.add("  type: device (GB300), %s storage\n", eps->storage == ksg::STORE_F64 ? "FP64" : "FP32-pair");
  if (ncv > 0 && eps->A) t.add("  %d columns of global length %d\n", ncv + 1, eps->A->m);
  t.add("  vector orthogonalization method: classical Gram-Schmidt, two passes (delayed)\n");
  // the DS as the reference's EPSView shows it: typed by EPSSetUp (or EPSSetFromOptions), untyped before
  DSType dtype = nullptr;
  if (eps->setup) dtype = ksg_eps_lanczos(eps) ? DSHEP : DSNHEP;
  else if (eps->ds) KSG_TRY(DSGetType(eps->ds, &dtype));
  t.add("DS Object: 1 MPI process\n");
  if (dtype) t.add("  type: %s\n", dtype);
  else t.add("  type not yet set\n");
  KSG_TRY(emit(v, t));
  eps->stobj.eps = eps;
  return STView(&eps->stobj, v);
}

// ---------------------------------------------------------------------------------------------------------------
// ST: the shift transformation with shift 0, owned by its EPS
// ---------------------------------------------------------------------------------------------------------------
extern "C" PetscErrorCode EPSGetST(EPS eps, ST *st) {
  KSG_CHECK(eps && st, PETSC_ERR_ARG_NULL, "Null argument");
  eps->stobj.eps = eps;
  *st = &eps->stobj;
  return 0;
}

extern "C" PetscErrorCode STSetType(ST st, STType type) {
  KSG_CHECK(st && type, PETSC_ERR_ARG_NULL, "Null argument");
  KSG_CHECK(!std::strcmp(type, STSHIFT), PETSC_ERR_SUP,
            "ST type %s is not provided: the Krylov-Schur path runs the shift transformation (STSHIFT)", type);
  st->typeset = 1;
  return 0;
}

extern "C" PetscErrorCode STGetType(ST st, STType *type) {
  KSG_CHECK(st && type, PETSC_ERR_ARG_NULL, "Null argument");
  *type = st->typeset ? STSHIFT : nullptr;  // no type until one is set, as the reference (stset.c:93)
  return 0;
}

extern "C" PetscErrorCode STSetShift(ST st, PetscScalar shift) {
  KSG_CHECK(st, PETSC_ERR_ARG_NULL, "Null ST");
  KSG_CHECK(shift == 0.0, PETSC_ERR_SUP, "Nonzero shifts (%g) are not provided", shift);
  return 0;
}

extern "C" PetscErrorCode STGetShift(ST st, PetscScalar *shift) {
  KSG_CHECK(st && shift, PETSC_ERR_ARG_NULL, "Null argument");
  *shift = 0.0;
  return 0;
}

extern "C" PetscErrorCode STGetNumMatrices(ST st, PetscInt *n) {
  KSG_CHECK(st && st->eps && n, PETSC_ERR_ARG_NULL, "Null argument");
  *n = st->eps->B ? 2 : 1;
  return 0;
}

// STView (stfunc.c): type, shift, number of matrices
extern "C" PetscErrorCode STView(ST st, PetscViewer v) {
  KSG_CHECK(st && st->eps, PETSC_ERR_ARG_NULL, "Null ST");
  if (!v) v = stdout_viewer();
  if (!v->ascii) return 0;
  Text t;
  t.add("ST Object: 1 MPI process\n");
  t.add(st->typeset ? "  type: shift\n" : "  type not yet set\n");
  t.add("  shift: 0.\n");
  t.add("  number of matrices: %d\n", st->eps->B ? 2 : 1);
  return emit(v, t);
}

// ---------------------------------------------------------------------------------------------------------------
// type queries and the options of other solver types (PetscTryMethod setters do nothing, PetscUseMethod getters fail)
// ---------------------------------------------------------------------------------------------------------------
const char *EPSPowerShiftTypes[] = {"CONSTANT", "RAYLEIGH", "WILKINSON", "EPSPowerShiftType", "EPS_POWER_SHIFT_",
                                    nullptr};
const char *EPSLanczosReorthogTypes[] = {"LOCAL", "FULL", "SELECTIVE", "PERIODIC", "PARTIAL", "DELAYED",
                                         "EPSLanczosReorthogType", "EPS_LANCZOS_REORTHOG_", nullptr};

namespace {
// the type name of an object of this library, by the cookie its struct begins with
const char *object_type(void *obj) {
  const unsigned c = *static_cast<const unsigned *>(obj);
  if (c == KSG_EPS_COOKIE) return static_cast<EPS>(obj)->type.c_str();
  if (c == KSG_ST_COOKIE) return STSHIFT;
  if (c == KSG_MAT_COOKIE) return static_cast<Mat>(obj)->dense ? "seqdense" : "seqaij";
  return "";
}
}  // namespace

extern "C" PetscErrorCode PetscObjectTypeCompare(void *obj, const char type[], PetscBool *same) {
  KSG_CHECK(same, PETSC_ERR_ARG_NULL, "Null argument");
  *same = (obj && type && !std::strcmp(object_type(obj), type)) ? PETSC_TRUE : PETSC_FALSE;
  return 0;
}

extern "C" PetscErrorCode PetscObjectTypeCompareAny(void *obj, PetscBool *match, const char type[], ...) {
  KSG_CHECK(match, PETSC_ERR_ARG_NULL, "Null argument");
  *match = PETSC_FALSE;
  va_list ap;
  va_start(ap, type);
  for (const char *t = type; t && t[0]; t = va_arg(ap, const char *))
    if (obj && !std::strcmp(object_type(obj), t)) *match = PETSC_TRUE;
  va_end(ap);
  return 0;
}

extern "C" PetscErrorCode EPSPowerSetShiftType(EPS eps, EPSPowerShiftType) {
  KSG_CHECK(eps, PETSC_ERR_ARG_NULL, "Null EPS");
  return 0;
}
extern "C" PetscErrorCode EPSPowerGetShiftType(EPS eps, EPSPowerShiftType *) {
  KSG_CHECK(eps, PETSC_ERR_ARG_NULL, "Null EPS");
  return ksg_set_error(PETSC_ERR_SUP, "EPSPowerGetShiftType: the EPS type is krylovschur, not power");
}
extern "C" PetscErrorCode EPSLanczosSetReorthog(EPS eps, EPSLanczosReorthogType) {
  KSG_CHECK(eps, PETSC_ERR_ARG_NULL, "Null EPS");
  return 0;
}
extern "C" PetscErrorCode EPSLanczosGetReorthog(EPS eps, EPSLanczosReorthogType *) {
  KSG_CHECK(eps, PETSC_ERR_ARG_NULL, "Null EPS");
  return ksg_set_error(PETSC_ERR_SUP, "EPSLanczosGetReorthog: the EPS type is krylovschur, not lanczos");
}
extern "C" PetscErrorCode EPSGDSetDoubleExpansion(EPS eps, PetscBool) {
  KSG_CHECK(eps, PETSC_ERR_ARG_NULL, "Null EPS");
  return 0;
}
extern "C" PetscErrorCode EPSGDGetDoubleExpansion(EPS eps, PetscBool *) {
  KSG_CHECK(eps, PETSC_ERR_ARG_NULL, "Null EPS");
  return ksg_set_error(PETSC_ERR_SUP, "EPSGDGetDoubleExpansion: the EPS type is krylovschur, not gd");
}

// EPSSetDeflationSpace (epsdefault.c / epssetup.c:523-560): the vectors are copied; EPSSetUp orthonormalises them
// on the device into constraint columns ahead of the Krylov basis (BVInsertConstraints), dropping dependent ones
extern "C" PetscErrorCode EPSSetDeflationSpace(EPS eps, PetscInt n, Vec v[]) {
  KSG_CHECK(eps, PETSC_ERR_ARG_NULL, "Null EPS");
  KSG_CHECK(n >= 0, PETSC_ERR_ARG_OUTOFRANGE, "Argument n cannot be negative");
  KSG_CHECK(n == 0 || v, PETSC_ERR_ARG_NULL, "Null vector array");
  int len = 0;
  for (PetscInt i = 0; i < n; ++i) {
    KSG_CHECK(v[i] && v[i]->a, PETSC_ERR_ARG_NULL, "Null vector %d", (int)i);
    KSG_CHECK(i == 0 || v[i]->n == len, PETSC_ERR_ARG_SIZ, "The deflation vectors must have one length");
    len = v[i]->n;
  }
  eps->defl.assign((size_t)n * len, 0.0);
  for (PetscInt i = 0; i < n; ++i) std::copy(v[i]->a, v[i]->a + len, eps->defl.begin() + (size_t)i * len);
  eps->ndefl = (int)n;
  eps->setup = 0;  // the next solve sets up again with the new constraints
  return 0;
}

// the shift of 0 runs no linear solver: its KSP handle is the ST's, and its iteration count 0
extern "C" PetscErrorCode STGetKSP(ST st, KSP *ksp) {
  KSG_CHECK(st && ksp, PETSC_ERR_ARG_NULL, "Null argument");
  *ksp = reinterpret_cast<KSP>(st);
  return 0;
}
extern "C" PetscErrorCode KSPGetTotalIterations(KSP ksp, PetscInt *its) {
  KSG_CHECK(ksp && its, PETSC_ERR_ARG_NULL, "Null argument");
  *its = 0;
  return 0;
}

// balancing, stopping test and track-all (epsopts.c): the defaults are this path's
const char *EPSBalanceTypes[] = {"NONE", "ONESIDE", "TWOSIDE", "USER", "EPSBalance", "EPS_BALANCE_", nullptr};

// EPSSetBalance (epsopts.c:1062-1092): the settings are stored and checked as the reference does.  A Hermitian
// problem is never balanced (epssetup.c:378-385); balancing a non-Hermitian one is refused by EPSSetUp.
extern "C" PetscErrorCode EPSSetBalance(EPS eps, EPSBalance bal, PetscInt its, PetscReal cutoff) {
  KSG_CHECK(eps, PETSC_ERR_ARG_NULL, "Null EPS");
  KSG_CHECK(bal == EPS_BALANCE_NONE || bal == EPS_BALANCE_ONESIDE || bal == EPS_BALANCE_TWOSIDE ||
                bal == EPS_BALANCE_USER, PETSC_ERR_ARG_OUTOFRANGE, "Invalid value of argument 'bal'");
  if (eps->balance != (int)bal) {
    eps->balance = bal;
    eps->setup = 0;
  }
  if (its == PETSC_DETERMINE) eps->balance_its = 5;
  else if (its != PETSC_CURRENT) {
    KSG_CHECK(its > 0, PETSC_ERR_ARG_OUTOFRANGE, "Illegal value of its. Must be > 0");
    eps->balance_its = its;
  }
  if (cutoff == (PetscReal)PETSC_DETERMINE) eps->balance_cutoff = 1e-8;
  else if (cutoff != (PetscReal)PETSC_CURRENT) {
    KSG_CHECK(cutoff > 0.0, PETSC_ERR_ARG_OUTOFRANGE, "Illegal value of cutoff. Must be > 0");
    eps->balance_cutoff = cutoff;
  }
  return 0;
}
extern "C" PetscErrorCode EPSGetBalance(EPS eps, EPSBalance *bal, PetscInt *its, PetscReal *cutoff) {
  KSG_CHECK(eps, PETSC_ERR_ARG_NULL, "Null EPS");
  if (bal) *bal = (EPSBalance)eps->balance;
  if (its) *its = eps->balance_its;
  if (cutoff) *cutoff = eps->balance_cutoff;
  return 0;
}
extern "C" PetscErrorCode EPSSetStoppingTest(EPS eps, EPSStop stop) {
  KSG_CHECK(eps, PETSC_ERR_ARG_NULL, "Null EPS");
  KSG_CHECK(stop == EPS_STOP_BASIC, PETSC_ERR_SUP, "Only EPS_STOP_BASIC is provided");
  return 0;
}
extern "C" PetscErrorCode EPSGetStoppingTest(EPS eps, EPSStop *stop) {
  KSG_CHECK(eps && stop, PETSC_ERR_ARG_NULL, "Null argument");
  *stop = EPS_STOP_BASIC;
  return 0;
}
extern "C" PetscErrorCode EPSSetTrackAll(EPS eps, PetscBool trackall) {
  KSG_CHECK(eps, PETSC_ERR_ARG_NULL, "Null EPS");
  eps->trackall = trackall ? 1 : 0;
  return 0;
}
extern "C" PetscErrorCode EPSGetTrackAll(EPS eps, PetscBool *trackall) {
  KSG_CHECK(eps && trackall, PETSC_ERR_ARG_NULL, "Null argument");
  *trackall = eps->trackall ? PETSC_TRUE : PETSC_FALSE;
  return 0;
}
extern "C" PetscErrorCode KSPSetTolerances(KSP ksp, PetscReal, PetscReal, PetscReal, PetscInt) {
  KSG_CHECK(ksp, PETSC_ERR_ARG_NULL, "Null KSP");
  return 0;  // the shift of 0 runs no linear solver
}
