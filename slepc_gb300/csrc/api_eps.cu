// api_eps.cu -- C API: errors, Mat, Vec and the EPS object with its device-resident Krylov-Schur driver.
//
// The restart loop is EPSSolve_KrylovSchur_Default (src/eps/impls/krylov/krylovschur/krylovschur.c:227-337):
//   factorise (SpMV + fused Gram-Schmidt pair per step, all launches asynchronous on the EPS stream)
//   -> projected problem, convergence, stopping test and restart sizes in one device kernel
//   -> one 64-byte control record read back per restart
//   -> thick restart V(:, nconv:k+l) = V(:, nconv:nv) Q, copy of the residual vector to column k+l.
// No scalar of a Krylov step crosses to the host.
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>
#include <strings.h>

#include <algorithm>
#include <cctype>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "internal.h"

using namespace ksg;

// ---------------------------------------------------------------------------------------------------------------
// errors
// ---------------------------------------------------------------------------------------------------------------
static thread_local char g_last_error[512] = "";

PetscErrorCode ksg_set_error(PetscErrorCode code, const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
  va_end(ap);
  return code;
}

extern "C" const char *PetscGB300LastError(void) { return g_last_error; }

extern "C" PetscErrorCode PetscInitialize(int *, char ***, const char[], const char[]) { return 0; }
extern "C" PetscErrorCode PetscFinalize(void) { return 0; }

static int g_argc = 0;
static char **g_argv = nullptr;
extern "C" PetscErrorCode SlepcInitialize(int *argc, char ***argv, const char[], const char[]) {
  if (argc && argv) {
    g_argc = *argc;
    g_argv = *argv;
  }
  return 0;
}
extern "C" PetscErrorCode SlepcFinalize(void) { return 0; }

// ---------------------------------------------------------------------------------------------------------------
// PETSc basics: PetscPrintf, the PetscCall error report, and the options database read from the argument list of
// SlepcInitialize (PetscOptionsGet*, petsc/src/sys/objects/options.c semantics: the last occurrence wins; an option
// name carries its dash, the prefix does not)
// ---------------------------------------------------------------------------------------------------------------
extern "C" void PetscGB300ReportError(PetscErrorCode ierr, const char *call, const char *file, int line) {
  std::fprintf(stderr, "[0]PETSC ERROR: %s returned %d at %s:%d\n[0]PETSC ERROR: %s\n", call, ierr, file, line,
               PetscGB300LastError());
}

extern "C" PetscErrorCode PetscPrintf(MPI_Comm, const char format[], ...) {
  KSG_CHECK(format, PETSC_ERR_ARG_NULL, "Null format");
  va_list ap;
  va_start(ap, format);
  std::vfprintf(stdout, format, ap);
  va_end(ap);
  std::fflush(stdout);
  return 0;
}

// the value of option -<pre><name without its dash>: nullptr if absent; *val the following argument, if it is one
static const char *opt_find(const char *pre, const char *name, const char **val) {
  *val = nullptr;
  if (!name || name[0] != '-') return nullptr;
  std::string key = std::string("-") + (pre ? pre : "") + (name + 1);
  const char *found = nullptr;
  for (int i = 1; i < g_argc; ++i) {
    if (!g_argv[i] || key != g_argv[i]) continue;
    found = g_argv[i];
    *val = nullptr;
    if (i + 1 < g_argc && g_argv[i + 1]) {
      const char *nx = g_argv[i + 1];
      const bool number = nx[0] == '-' && (std::isdigit((unsigned char)nx[1]) || nx[1] == '.');
      if (nx[0] != '-' || number) *val = nx;
    }
  }
  return found;
}

extern "C" PetscErrorCode PetscOptionsHasName(PetscOptions, const char pre[], const char name[], PetscBool *set) {
  KSG_CHECK(name && set, PETSC_ERR_ARG_NULL, "Null argument");
  const char *v;
  *set = opt_find(pre, name, &v) ? PETSC_TRUE : PETSC_FALSE;
  return 0;
}

extern "C" PetscErrorCode PetscOptionsGetInt(PetscOptions, const char pre[], const char name[], PetscInt *ivalue,
                                             PetscBool *set) {
  KSG_CHECK(name && ivalue, PETSC_ERR_ARG_NULL, "Null argument");
  const char *v;
  const char *f = opt_find(pre, name, &v);
  if (set) *set = PETSC_FALSE;
  if (!f) return 0;
  KSG_CHECK(v, PETSC_ERR_ARG_WRONG, "Missing value for option %s", f);
  char *end = nullptr;
  const long x = std::strtol(v, &end, 10);
  KSG_CHECK(end && *end == 0, PETSC_ERR_ARG_WRONG, "Input string %s has no integer value", v);
  *ivalue = (PetscInt)x;
  if (set) *set = PETSC_TRUE;
  return 0;
}

extern "C" PetscErrorCode PetscOptionsGetReal(PetscOptions, const char pre[], const char name[], PetscReal *dvalue,
                                              PetscBool *set) {
  KSG_CHECK(name && dvalue, PETSC_ERR_ARG_NULL, "Null argument");
  const char *v;
  const char *f = opt_find(pre, name, &v);
  if (set) *set = PETSC_FALSE;
  if (!f) return 0;
  KSG_CHECK(v, PETSC_ERR_ARG_WRONG, "Missing value for option %s", f);
  char *end = nullptr;
  const double x = std::strtod(v, &end);
  KSG_CHECK(end && *end == 0, PETSC_ERR_ARG_WRONG, "Input string %s has no numeric value", v);
  *dvalue = x;
  if (set) *set = PETSC_TRUE;
  return 0;
}

extern "C" PetscErrorCode PetscOptionsGetScalar(PetscOptions o, const char pre[], const char name[],
                                                PetscScalar *dvalue, PetscBool *set) {
  return PetscOptionsGetReal(o, pre, name, dvalue, set);
}

extern "C" PetscErrorCode PetscOptionsGetBool(PetscOptions, const char pre[], const char name[], PetscBool *ivalue,
                                              PetscBool *set) {
  KSG_CHECK(name, PETSC_ERR_ARG_NULL, "Null argument");
  const char *v;
  const char *f = opt_find(pre, name, &v);
  if (set) *set = PETSC_FALSE;
  if (!f) return 0;
  PetscBool b = PETSC_TRUE;  // the bare option means true
  if (v) {
    std::string t(v);
    for (char &c : t) c = (char)std::tolower((unsigned char)c);
    if (t == "0" || t == "false" || t == "no" || t == "off") b = PETSC_FALSE;
    else KSG_CHECK(t == "1" || t == "true" || t == "yes" || t == "on", PETSC_ERR_ARG_WRONG,
                   "Unknown logical value: %s", v);
  }
  if (ivalue) *ivalue = b;
  if (set) *set = PETSC_TRUE;
  return 0;
}

extern "C" PetscErrorCode PetscOptionsGetString(PetscOptions, const char pre[], const char name[], char string[],
                                                size_t len, PetscBool *set) {
  KSG_CHECK(name && string, PETSC_ERR_ARG_NULL, "Null argument");
  const char *v;
  const char *f = opt_find(pre, name, &v);
  if (set) *set = PETSC_FALSE;
  if (!f) return 0;
  if (len > 0) {
    std::strncpy(string, v ? v : "", len - 1);
    string[len - 1] = 0;
  }
  if (set) *set = PETSC_TRUE;
  return 0;
}

// ---------------------------------------------------------------------------------------------------------------
// random vectors: splitmix64 uniform in [-1, 1), counter-based so that any column can be regenerated
// ---------------------------------------------------------------------------------------------------------------
PetscErrorCode ksg_random_fill(double *host, int n, unsigned long long seed, unsigned long long stream_index) {
  unsigned long long base = seed ^ (0xD1B54A32D192ED03ULL * (stream_index + 1));
  for (int i = 0; i < n; ++i) {
    unsigned long long z = base + (unsigned long long)(i + 1) * 0x9E3779B97F4A7C15ULL;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    z ^= z >> 31;
    host[i] = (double)(z >> 11) * (2.0 / 9007199254740992.0) - 1.0;
  }
  return 0;
}

// ---------------------------------------------------------------------------------------------------------------
// Mat
// ---------------------------------------------------------------------------------------------------------------
extern "C" PetscErrorCode MatCreateSeqAIJWithArrays(MPI_Comm, PetscInt m, PetscInt n, PetscInt i[], PetscInt j[],
                                                    PetscScalar a[], Mat *A) {
  KSG_CHECK(A, PETSC_ERR_ARG_NULL, "Null Mat pointer");
  KSG_CHECK(m >= 0 && n >= 0, PETSC_ERR_ARG_OUTOFRANGE, "Negative dimension");
  KSG_CHECK(i && (i[m] == 0 || (j && a)), PETSC_ERR_ARG_NULL, "Null CSR array");
  KSG_CHECK(i[0] == 0, PETSC_ERR_ARG_WRONG, "i (row pointers) must start with 0");
  for (int r = 0; r < m; ++r)
    KSG_CHECK(i[r + 1] >= i[r], PETSC_ERR_ARG_WRONG, "Row pointers must be nondecreasing (row %d)", r);
  // entries checked in parallel; the first failing row (in row order) is the one reported
  int bad = m;
#pragma omp parallel for reduction(min : bad) schedule(static)
  for (int r = 0; r < m; ++r)
    for (int p = i[r]; p < i[r + 1]; ++p)
      if (!(j[p] >= 0 && j[p] < n) || !isfinite(a[p])) {
        bad = std::min(bad, r);
        break;
      }
  if (bad < m)
    for (int p = i[bad]; p < i[bad + 1]; ++p) {
      KSG_CHECK(j[p] >= 0 && j[p] < n, PETSC_ERR_ARG_OUTOFRANGE, "Column index %d out of range in row %d", j[p], bad);
      KSG_CHECK(isfinite(a[p]), PETSC_ERR_ARG_WRONG, "Matrix entry (%d,%d) is not finite", bad, j[p]);
    }
  Mat M = new _p_Mat();
  M->m = m;
  M->n = n;
  M->ai = i;
  M->aj = j;
  M->aa = a;
  M->nnz = i[m];
  *A = M;
  return 0;
}

extern "C" PetscErrorCode MatCreateSeqDense(MPI_Comm, PetscInt m, PetscInt n, PetscScalar data[], Mat *A) {
  KSG_CHECK(A, PETSC_ERR_ARG_NULL, "Null Mat pointer");
  KSG_CHECK(m >= 0 && n >= 0, PETSC_ERR_ARG_OUTOFRANGE, "Negative dimension");
  Mat M = new _p_Mat();
  M->m = m;
  M->n = n;
  M->dense = 1;
  M->lda = m > 0 ? m : 1;
  if (data) M->data = data;
  else {
    M->dbuf.assign((size_t)M->lda * (n > 0 ? n : 1), 0.0);
    M->data = M->dbuf.data();
  }
  *A = M;
  return 0;
}

extern "C" PetscErrorCode MatDenseGetArray(Mat A, PetscScalar **array) {
  KSG_CHECK(A && A->dense, PETSC_ERR_ARG_WRONG, "Not a dense Mat");
  *array = A->data;
  return 0;
}
extern "C" PetscErrorCode MatDenseRestoreArray(Mat A, PetscScalar **array) {
  if (array) *array = nullptr;
  return 0;
}
extern "C" PetscErrorCode MatDenseGetLDA(Mat A, PetscInt *lda) {
  KSG_CHECK(A && A->dense, PETSC_ERR_ARG_WRONG, "Not a dense Mat");
  *lda = A->lda;
  return 0;
}
extern "C" PetscErrorCode MatGetSize(Mat A, PetscInt *m, PetscInt *n) {
  KSG_CHECK(A, PETSC_ERR_ARG_NULL, "Null Mat");
  if (m) *m = A->m;
  if (n) *n = A->n;
  return 0;
}
extern "C" PetscErrorCode MatGetValue(Mat A, PetscInt row, PetscInt col, PetscScalar *v) {
  KSG_CHECK(A && v, PETSC_ERR_ARG_NULL, "Null argument");
  KSG_CHECK(row >= 0 && row < A->m && col >= 0 && col < A->n, PETSC_ERR_ARG_OUTOFRANGE, "Index out of range");
  if (A->dense) {
    *v = A->data[row + (size_t)col * A->lda];
    return 0;
  }
  *v = 0.0;
  for (int p = A->ai[row]; p < A->ai[row + 1]; ++p)
    if (A->aj[p] == col) *v += A->aa[p];
  return 0;
}

PetscErrorCode ksg_mat_upload(Mat A) {
  if (A->device_ready) return 0;
  KSG_CHECK(!A->dense, PETSC_ERR_SUP, "Operator must be an AIJ (CSR) matrix");
  KSG_CUDA(A->d_rp.alloc(A->m + 1));
  KSG_CUDA(A->d_ci.alloc(A->nnz > 0 ? A->nnz : 1));
  KSG_CUDA(A->d_va.alloc(A->nnz > 0 ? A->nnz : 1));
  KSG_CUDA(cudaMemcpy(A->d_rp.p, A->ai, sizeof(int) * (A->m + 1), cudaMemcpyHostToDevice));
  if (A->nnz > 0) {
    KSG_CUDA(cudaMemcpy(A->d_ci.p, A->aj, sizeof(int) * A->nnz, cudaMemcpyHostToDevice));
    KSG_CUDA(cudaMemcpy(A->d_va.p, A->aa, sizeof(double) * A->nnz, cudaMemcpyHostToDevice));
  }
  // long rows -> segments (host side, once per matrix)
  {
    std::vector<int> sr, sb, se, lr, lf;
    for (int r = 0; r < A->m; ++r) {
      const int p0 = A->ai[r], p1 = A->ai[r + 1];
      if (p1 - p0 <= LONG_ROW_T) continue;
      lr.push_back(r);
      lf.push_back((int)sr.size());
      for (int p = p0; p < p1; p += LONG_SEG) {
        sr.push_back(r);
        sb.push_back(p);
        se.push_back(std::min(p1, p + LONG_SEG));
      }
    }
    A->n_long = (int)lr.size();
    A->n_seg = (int)sr.size();
    if (A->n_long > 0) {
      lf.push_back(A->n_seg);
      KSG_CUDA(A->d_seg_row.alloc(A->n_seg));
      KSG_CUDA(A->d_seg_beg.alloc(A->n_seg));
      KSG_CUDA(A->d_seg_end.alloc(A->n_seg));
      KSG_CUDA(A->d_lrow.alloc(A->n_long));
      KSG_CUDA(A->d_lfirst.alloc(A->n_long + 1));
      KSG_CUDA(cudaMemcpy(A->d_seg_row.p, sr.data(), sizeof(int) * A->n_seg, cudaMemcpyHostToDevice));
      KSG_CUDA(cudaMemcpy(A->d_seg_beg.p, sb.data(), sizeof(int) * A->n_seg, cudaMemcpyHostToDevice));
      KSG_CUDA(cudaMemcpy(A->d_seg_end.p, se.data(), sizeof(int) * A->n_seg, cudaMemcpyHostToDevice));
      KSG_CUDA(cudaMemcpy(A->d_lrow.p, lr.data(), sizeof(int) * A->n_long, cudaMemcpyHostToDevice));
      KSG_CUDA(cudaMemcpy(A->d_lfirst.p, lf.data(), sizeof(int) * (A->n_long + 1), cudaMemcpyHostToDevice));
    }
  }
  A->device_ready = 1;
  return 0;
}

PetscErrorCode ksg_mat_upload_pairs(Mat A) {
  KSG_TRY(ksg_mat_upload(A));
  if (A->d_va2.p || A->nnz == 0) return 0;
  // split on the device from the FP64 values already there (hi = fl32(v), lo = fl32(v - hi)); the solver streams do
  // not order themselves after the legacy stream, hence the synchronisation
  KSG_CUDA(A->d_va2.alloc(A->nnz));
  KSG_CUDA(launch_f64_to_pair(A->d_va.p, A->d_va2.p, A->nnz, 0));
  KSG_CUDA(cudaStreamSynchronize(0));
  return 0;
}

void *ksg_col(void *V, long long ldv, int j, int storage) {
  return static_cast<char *>(V) + (size_t)j * (size_t)ldv * ksg_entry_bytes(storage);
}

PetscErrorCode ksg_mat_upload_f32(Mat A) {
  KSG_TRY(ksg_mat_upload(A));
  if (A->d_va32.p || A->nnz == 0) return 0;
  KSG_CUDA(A->d_va32.alloc(A->nnz));
  KSG_CUDA(launch_f64_to_f32(A->d_va.p, A->d_va32.p, A->nnz, 0));
  KSG_CUDA(cudaStreamSynchronize(0));
  return 0;
}

PetscErrorCode ksg_put_column(void *dst, const double *src, int n, int storage, cudaStream_t s) {
  if (storage == STORE_F64) {
    KSG_CUDA(cudaMemcpyAsync(dst, src, sizeof(double) * n, cudaMemcpyHostToDevice, s));
    return 0;
  }
  if (storage == STORE_F32) {
    std::vector<float> h(n);
    for (int i = 0; i < n; ++i) h[i] = (float)src[i];
    KSG_CUDA(cudaMemcpyAsync(dst, h.data(), sizeof(float) * n, cudaMemcpyHostToDevice, s));
    KSG_CUDA(cudaStreamSynchronize(s));
    return 0;
  }
  std::vector<float2> h(n);
  for (int i = 0; i < n; ++i) {
    const float hi = (float)src[i];
    h[i] = make_float2(hi, (float)(src[i] - (double)hi));
  }
  KSG_CUDA(cudaMemcpyAsync(dst, h.data(), sizeof(float2) * n, cudaMemcpyHostToDevice, s));
  KSG_CUDA(cudaStreamSynchronize(s));
  return 0;
}

PetscErrorCode ksg_get_column(double *dst, const void *src, int n, int storage, cudaStream_t s) {
  if (storage == STORE_F64) {
    KSG_CUDA(cudaMemcpyAsync(dst, src, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
    KSG_CUDA(cudaStreamSynchronize(s));
    return 0;
  }
  if (storage == STORE_F32) {
    std::vector<float> h(n);
    KSG_CUDA(cudaMemcpyAsync(h.data(), src, sizeof(float) * n, cudaMemcpyDeviceToHost, s));
    KSG_CUDA(cudaStreamSynchronize(s));
    for (int i = 0; i < n; ++i) dst[i] = (double)h[i];
    return 0;
  }
  std::vector<float2> h(n);
  KSG_CUDA(cudaMemcpyAsync(h.data(), src, sizeof(float2) * n, cudaMemcpyDeviceToHost, s));
  KSG_CUDA(cudaStreamSynchronize(s));
  for (int i = 0; i < n; ++i) dst[i] = (double)h[i].x + (double)h[i].y;
  return 0;
}

double ksg_mat_norm_inf(Mat A) {
  if (A->norm_inf >= 0.0) return A->norm_inf;
  double mx = 0.0;
  if (A->dense) {
    for (int r = 0; r < A->m; ++r) {
      double s = 0.0;
      for (int c = 0; c < A->n; ++c) s += fabs(A->data[r + (size_t)c * A->lda]);
      mx = std::max(mx, s);
    }
  } else {
    // rows in parallel; each row summed in order, so the maximum is the same as a sequential pass
#pragma omp parallel for reduction(max : mx) schedule(static)
    for (int r = 0; r < A->m; ++r) {
      double s = 0.0;
      for (int p = A->ai[r]; p < A->ai[r + 1]; ++p) s += fabs(A->aa[p]);
      mx = std::max(mx, s);
    }
  }
  A->norm_inf = mx;
  return mx;
}

extern "C" PetscErrorCode MatNorm(Mat A, NormType type, PetscReal *nrm) {
  KSG_CHECK(A && nrm, PETSC_ERR_ARG_NULL, "Null argument");
  if (type == NORM_INFINITY) {
    *nrm = ksg_mat_norm_inf(A);
    return 0;
  }
  if (type == NORM_FROBENIUS) {
    double s = 0.0;
    if (A->dense) {
      for (int c = 0; c < A->n; ++c)
        for (int r = 0; r < A->m; ++r) s += A->data[r + (size_t)c * A->lda] * A->data[r + (size_t)c * A->lda];
    } else {
      for (long long p = 0; p < A->nnz; ++p) s += A->aa[p] * A->aa[p];
    }
    *nrm = sqrt(s);
    return 0;
  }
  if (type == NORM_1) {
    std::vector<double> col(A->n, 0.0);
    if (A->dense) {
      for (int c = 0; c < A->n; ++c)
        for (int r = 0; r < A->m; ++r) col[c] += fabs(A->data[r + (size_t)c * A->lda]);
    } else {
      for (long long p = 0; p < A->nnz; ++p) col[A->aj[p]] += fabs(A->aa[p]);
    }
    *nrm = col.empty() ? 0.0 : *std::max_element(col.begin(), col.end());
    return 0;
  }
  return ksg_set_error(PETSC_ERR_SUP, "MatNorm: unsupported norm type");
}

extern "C" PetscErrorCode MatMult(Mat A, Vec x, Vec y) {
  KSG_CHECK(A && x && y, PETSC_ERR_ARG_NULL, "Null argument");
  KSG_CHECK(!A->empty, PETSC_ERR_ARG_WRONGSTATE, "The Mat holds no data (MatCreate without MatLoad)");
  KSG_CHECK(x->n == A->n && y->n == A->m, PETSC_ERR_ARG_SIZ, "Nonconforming sizes");
  if (A->dense) return ksg_set_error(PETSC_ERR_SUP, "MatMult on a dense Mat is not provided");
  KSG_TRY(ksg_mat_upload(A));
  DBuf<double> dx, dy;
  KSG_CUDA(dx.alloc(A->n > 0 ? A->n : 1));
  KSG_CUDA(dy.alloc(A->m > 0 ? A->m : 1));
  KSG_CUDA(cudaMemcpy(dx.p, x->a, sizeof(double) * A->n, cudaMemcpyHostToDevice));
  const int lanes = spmv_lanes_for(A->m > 0 ? (double)A->nnz / A->m : 1.0);
  KSG_CUDA(launch_spmv(A->d_rp.p, A->d_ci.p, A->d_va.p, dx.p, dy.p, A->m, lanes, nullptr, 1.0, 0));
  KSG_CUDA(cudaMemcpy(y->a, dy.p, sizeof(double) * A->m, cudaMemcpyDeviceToHost));
  return 0;
}

extern "C" PetscErrorCode MatCreateVecs(Mat A, Vec *right, Vec *left) {
  KSG_CHECK(A, PETSC_ERR_ARG_NULL, "Null Mat");
  if (right) KSG_TRY(VecCreateSeq(0, A->n, right));
  if (left) KSG_TRY(VecCreateSeq(0, A->m, left));
  return 0;
}

extern "C" PetscErrorCode MatDestroy(Mat *A) {
  if (!A || !*A) return 0;
  if (--(*A)->refs <= 0) delete *A;
  *A = nullptr;
  return 0;
}

// ---------------------------------------------------------------------------------------------------------------
// Vec
// ---------------------------------------------------------------------------------------------------------------
extern "C" PetscErrorCode VecCreateSeq(MPI_Comm, PetscInt n, Vec *v) {
  KSG_CHECK(v, PETSC_ERR_ARG_NULL, "Null Vec pointer");
  KSG_CHECK(n >= 0, PETSC_ERR_ARG_OUTOFRANGE, "Negative size");
  Vec V = new _p_Vec();
  V->n = n;
  V->own.assign(n > 0 ? n : 1, 0.0);
  V->a = V->own.data();
  *v = V;
  return 0;
}
extern "C" PetscErrorCode VecCreateSeqWithArray(MPI_Comm, PetscInt, PetscInt n, const PetscScalar array[], Vec *v) {
  KSG_CHECK(v, PETSC_ERR_ARG_NULL, "Null Vec pointer");
  KSG_CHECK(n >= 0, PETSC_ERR_ARG_OUTOFRANGE, "Negative size");
  Vec V = new _p_Vec();
  V->n = n;
  if (array) V->a = const_cast<double *>(array);
  else {
    V->own.assign(n > 0 ? n : 1, 0.0);
    V->a = V->own.data();
  }
  *v = V;
  return 0;
}
extern "C" PetscErrorCode VecDuplicate(Vec v, Vec *newv) { return VecCreateSeq(0, v->n, newv); }
extern "C" PetscErrorCode VecGetSize(Vec v, PetscInt *n) {
  KSG_CHECK(v && n, PETSC_ERR_ARG_NULL, "Null argument");
  *n = v->n;
  return 0;
}
extern "C" PetscErrorCode VecGetArray(Vec v, PetscScalar **a) {
  KSG_CHECK(v && a, PETSC_ERR_ARG_NULL, "Null argument");
  *a = v->a;
  return 0;
}
extern "C" PetscErrorCode VecRestoreArray(Vec, PetscScalar **a) {
  if (a) *a = nullptr;
  return 0;
}
extern "C" PetscErrorCode VecGetArrayRead(Vec v, const PetscScalar **a) {
  KSG_CHECK(v && a, PETSC_ERR_ARG_NULL, "Null argument");
  *a = v->a;
  return 0;
}
extern "C" PetscErrorCode VecRestoreArrayRead(Vec, const PetscScalar **a) {
  if (a) *a = nullptr;
  return 0;
}
extern "C" PetscErrorCode VecSet(Vec v, PetscScalar alpha) {
  KSG_CHECK(v, PETSC_ERR_ARG_NULL, "Null Vec");
  for (int i = 0; i < v->n; ++i) v->a[i] = alpha;
  return 0;
}
extern "C" PetscErrorCode VecCopy(Vec x, Vec y) {
  KSG_CHECK(x && y && x->n == y->n, PETSC_ERR_ARG_SIZ, "Nonconforming vectors");
  memmove(y->a, x->a, sizeof(double) * x->n);
  return 0;
}
extern "C" PetscErrorCode VecScale(Vec v, PetscScalar alpha) {
  KSG_CHECK(v, PETSC_ERR_ARG_NULL, "Null Vec");
  for (int i = 0; i < v->n; ++i) v->a[i] *= alpha;
  return 0;
}
extern "C" PetscErrorCode VecAXPY(Vec y, PetscScalar alpha, Vec x) {
  KSG_CHECK(x && y && x->n == y->n, PETSC_ERR_ARG_SIZ, "Nonconforming vectors");
  for (int i = 0; i < x->n; ++i) y->a[i] += alpha * x->a[i];
  return 0;
}
extern "C" PetscErrorCode VecDot(Vec x, Vec y, PetscScalar *val) {
  KSG_CHECK(x && y && val && x->n == y->n, PETSC_ERR_ARG_SIZ, "Nonconforming vectors");
  double s = 0.0;
  for (int i = 0; i < x->n; ++i) s += x->a[i] * y->a[i];
  *val = s;
  return 0;
}
extern "C" PetscErrorCode VecNorm(Vec v, NormType type, PetscReal *nrm) {
  KSG_CHECK(v && nrm, PETSC_ERR_ARG_NULL, "Null argument");
  double r = 0.0;
  if (type == NORM_2 || type == NORM_FROBENIUS) {
    for (int i = 0; i < v->n; ++i) r += v->a[i] * v->a[i];
    r = sqrt(r);
  } else if (type == NORM_1) {
    for (int i = 0; i < v->n; ++i) r += fabs(v->a[i]);
  } else if (type == NORM_INFINITY) {
    for (int i = 0; i < v->n; ++i) r = std::max(r, fabs(v->a[i]));
  } else return ksg_set_error(PETSC_ERR_SUP, "VecNorm: unsupported norm type");
  *nrm = r;
  return 0;
}
extern "C" PetscErrorCode VecDestroy(Vec *v) {
  if (!v || !*v) return 0;
  delete *v;
  *v = nullptr;
  return 0;
}

// ---------------------------------------------------------------------------------------------------------------
// shared Gram-Schmidt helper: orthonormalise V[:, j] against V[:, 0:j] with CGS passes (REFINE_IFNEEDED when
// refine == 0, two passes when refine == 2, one pass plus explicit norm when refine == 1)
// ---------------------------------------------------------------------------------------------------------------
size_t ksg_part_stride(int ld) { return (size_t)2 * ld + 8; }
size_t ksg_part_blocks(int n) { return (size_t)std::max(gs_dot_blocks(n), gs_update_blocks(n)); }

PetscErrorCode ksg_orthonormalize_column(void *V, long long ldv, int n, int j, double *coef, float2 *part,
                                         int pstride, KrylovState *st, int arith, cudaStream_t s, double *nrm,
                                         int *lindep, int refine, int storage, const GTArgs *tc) {
  StepArgs a = {};
  a.tc = tc;
  a.V = V;
  a.ldv = ldv;
  a.n = n;
  a.J = j;
  a.j = j;
  a.hermitian = 1;
  a.U = ksg_col(V, ldv, j, storage);
  a.W = nullptr;
  a.eta = 0.7071;
  a.coef = coef;
  a.part = part;
  a.pstride = pstride;
  a.st = st;
  // refine: 0 IFNEEDED (up to 3 passes, bvorthog.c:176-187), 1 NEVER (one pass), 2 ALWAYS (two passes)
  const int passes_max = (refine == 2) ? 2 : (refine == 1 ? 1 : 3);
  double total = 1.0;
  int ld = 0;
  for (int pass = 0; pass < passes_max; ++pass) {
    KSG_CUDA(launch_segment_begin(st, j, j, s));
    KSG_CUDA(launch_gs_dot(a, 1, GS_ORTHO, arith, s, storage));
    KSG_CUDA(launch_gs_update(a, 1, GS_ORTHO, arith, s, storage));
    KrylovState h;
    KSG_CUDA(cudaMemcpyAsync(&h, st, sizeof(h), cudaMemcpyDeviceToHost, s));
    KSG_CUDA(cudaStreamSynchronize(s));
    if (h.breakdown) {
      total = 0.0;
      ld = 1;
      break;
    }
    const double nu = 1.0 / h.invnu;  // norm kept by this pass (the pass leaves the vector normalised)
    total *= nu;
    const int kept = nu >= 0.7071 * h.onorm;
    if (refine == 1) break;
    if (refine == 0) {
      if (kept) break;
      if (pass == passes_max - 1) ld = 1;
    }
    if (refine == 2 && pass == 1) ld = !kept;
  }
  if (nrm) *nrm = total;
  if (lindep) *lindep = ld;
  return 0;
}

// ---------------------------------------------------------------------------------------------------------------
// EPS
// ---------------------------------------------------------------------------------------------------------------
// factorisation segments replay from CUDA graphs by default up to this many rows (EPSGB300SetGraphCapture)
constexpr int kGraphMaxRows = 262144;

static void eps_clear_graphs(EPS eps) {
  for (auto &kv : eps->seg_graphs)
    if (kv.second.exec) cudaGraphExecDestroy(kv.second.exec);
  eps->seg_graphs.clear();
}

static PetscErrorCode eps_free_device(EPS eps) {
  eps_clear_graphs(eps);
  eps->V.release();
  eps->d.release();
  eps->e.release();
  eps->H.release();
  eps->Q.release();
  eps->X.release();
  eps->eigr.release();
  eps->eigi.release();
  eps->errest.release();
  eps->coef.release();
  eps->work.release();
  eps->dsf.release();
  eps->seg_part.release();
  eps->xvec.release();
  eps->d_perm.release();
  eps->vexp.release();
  eps->gtpart.release();
  eps->gterr.release();
  eps->gs_tc_on = 0;
  eps->xvec_valid = 0;
  eps->rtc.release();
  eps->part.release();
  eps->st.release();
  eps->ctl.release();
  if (eps->h_ctl) {
    cudaFreeHost(eps->h_ctl);
    eps->h_ctl = nullptr;
  }
  eps->setup = 0;
  return 0;
}

extern "C" PetscErrorCode EPSCreate(MPI_Comm, EPS *outeps) {
  KSG_CHECK(outeps, PETSC_ERR_ARG_NULL, "Null EPS pointer");
  EPS eps = new _p_EPS();
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) dev = 0;
  eps->device = dev;
  *outeps = eps;
  return 0;
}

extern "C" PetscErrorCode EPSReset(EPS eps) {
  KSG_CHECK(eps, PETSC_ERR_ARG_NULL, "Null EPS");
  eps_free_device(eps);
  eps->solved = 0;
  eps->nconv = 0;
  return 0;
}

// the operator the solver iterates on is A itself or an EPS-owned scaled copy (generalised problems)
static void eps_drop_operator(EPS e) {
  if (e->op && e->op != e->A) MatDestroy(&e->op);
  e->op = nullptr;
}

// EPSMonitorSet / EPSMonitorCancel (epsmon.c:62-130): up to 5 monitors, called after every restart
extern "C" PetscErrorCode EPSMonitorSet(EPS eps, EPSMonitorFn *monitor, void *mctx, PetscCtxDestroyFn *monitordestroy) {
  KSG_CHECK(eps, PETSC_ERR_ARG_NULL, "Null EPS");
  KSG_CHECK(eps->mon.size() < 5, PETSC_ERR_ARG_OUTOFRANGE, "Too many EPS monitors set");
  if (!monitor) return 0;
  eps->mon.push_back(monitor);
  eps->mon_ctx.push_back(mctx);
  eps->mon_destroy.push_back(monitordestroy);
  return 0;
}
extern "C" PetscErrorCode EPSMonitorCancel(EPS eps) {
  KSG_CHECK(eps, PETSC_ERR_ARG_NULL, "Null EPS");
  PetscErrorCode first = 0;
  for (size_t i = 0; i < eps->mon.size(); ++i)
    if (eps->mon_destroy[i]) {
      void *c = eps->mon_ctx[i];
      const PetscErrorCode e = eps->mon_destroy[i](&c);
      if (e && !first) first = e;
    }
  eps->mon.clear();
  eps->mon_ctx.clear();
  eps->mon_destroy.clear();
  return first;
}

// EPSMonitor (epsmon.c:40-48) after a restart: the nest current Ritz values (operator scaling undone) and their error
// estimates, read from the device
static PetscErrorCode eps_run_monitors(EPS eps, int its, int nconv, int nest, cudaStream_t s) {
  std::vector<double> er(nest), ei(nest), es(nest);
  KSG_CUDA(cudaMemcpyAsync(er.data(), eps->eigr.p, sizeof(double) * nest, cudaMemcpyDeviceToHost, s));
  KSG_CUDA(cudaMemcpyAsync(ei.data(), eps->eigi.p, sizeof(double) * nest, cudaMemcpyDeviceToHost, s));
  KSG_CUDA(cudaMemcpyAsync(es.data(), eps->errest.p, sizeof(double) * nest, cudaMemcpyDeviceToHost, s));
  KSG_CUDA(cudaStreamSynchronize(s));
  for (int i = 0; i < nest; ++i) {
    er[i] /= eps->opscale;
    ei[i] = ksg_eps_hermitian(eps) && eps->extraction != EPS_HARMONIC ? 0.0 : ei[i] / eps->opscale;
  }
  for (size_t m = 0; m < eps->mon.size(); ++m)
    KSG_TRY(eps->mon[m](eps, its, nconv, er.data(), ei.data(), es.data(), nest, eps->mon_ctx[m]));
  return 0;
}

extern "C" PetscErrorCode EPSDestroy(EPS *eps) {
  if (!eps || !*eps) return 0;
  EPS e = *eps;
  EPSMonitorCancel(e);
  if (e->device >= 0) cudaSetDevice(e->device);
  eps_free_device(e);
  for (cudaEvent_t ev : e->ev_pool) cudaEventDestroy(ev);
  for (cudaEvent_t ev : e->ev_solve)
    if (ev) cudaEventDestroy(ev);
  if (e->bv) BVDestroy(&e->bv);
  if (e->ds) DSDestroy(&e->ds);
  if (e->stream) cudaStreamDestroy(e->stream);
  eps_drop_operator(e);
  if (e->A) MatDestroy(&e->A);
  if (e->B) MatDestroy(&e->B);
  delete e;
  *eps = nullptr;
  return 0;
}

extern "C" PetscErrorCode EPSSetType(EPS eps, EPSType type) {
  KSG_CHECK(eps && type, PETSC_ERR_ARG_NULL, "Null argument");
  KSG_CHECK(strcmp(type, EPSKRYLOVSCHUR) == 0, PETSC_ERR_SUP, "Only EPSKRYLOVSCHUR is provided (requested %s)", type);
  eps->type = type;
  return 0;
}
extern "C" PetscErrorCode EPSGetType(EPS eps, EPSType *type) {
  KSG_CHECK(eps && type, PETSC_ERR_ARG_NULL, "Null argument");
  *type = EPSKRYLOVSCHUR;
  return 0;
}
// EPSSetOperators (epssetup.c:440-500): A, and B for a generalised problem (sizes checked as there)
extern "C" PetscErrorCode EPSSetOperators(EPS eps, Mat A, Mat B) {
  KSG_CHECK(eps && A, PETSC_ERR_ARG_NULL, "Null argument");
  KSG_CHECK(!A->empty, PETSC_ERR_ARG_WRONGSTATE, "Not for unassembled matrix (A)");
  KSG_CHECK(A->m == A->n, PETSC_ERR_ARG_WRONG, "A does not have equal row and column sizes (%d, %d)", A->m, A->n);
  if (B) {
    KSG_CHECK(!B->empty, PETSC_ERR_ARG_WRONGSTATE, "Not for unassembled matrix (B)");
    KSG_CHECK(B->m == B->n, PETSC_ERR_ARG_WRONG, "B is a non-square matrix (%d rows, %d cols)", B->m, B->n);
    KSG_CHECK(A->m == B->m, PETSC_ERR_ARG_INCOMP, "Dimensions of A and B do not match (%d, %d)", A->m, B->m);
    B->refs++;
  }
  A->refs++;
  eps_drop_operator(eps);
  if (eps->A) MatDestroy(&eps->A);
  if (eps->B) MatDestroy(&eps->B);
  eps->A = A;
  eps->B = B;
  eps->nrma = eps->nrmb = 0.0;
  eps->setup = 0;
  eps->solved = 0;
  return 0;
}
extern "C" PetscErrorCode EPSGetOperators(EPS eps, Mat *A, Mat *B) {
  KSG_CHECK(eps, PETSC_ERR_ARG_NULL, "Null EPS");
  if (A) *A = eps->A;
  if (B) *B = eps->B;
  return 0;
}
extern "C" PetscErrorCode EPSSetProblemType(EPS eps, EPSProblemType type) {
  KSG_CHECK(eps, PETSC_ERR_ARG_NULL, "Null EPS");
  KSG_CHECK(type == EPS_HEP || type == EPS_NHEP || type == EPS_GHEP || type == EPS_GNHEP, PETSC_ERR_SUP,
            "Only EPS_HEP, EPS_NHEP, EPS_GHEP and EPS_GNHEP are provided");
  eps->problem = type;
  eps->setup = 0;
  eps->solved = 0;
  return 0;
}
extern "C" PetscErrorCode EPSGetProblemType(EPS eps, EPSProblemType *type) {
  KSG_CHECK(eps && type, PETSC_ERR_ARG_NULL, "Null argument");
  *type = (EPSProblemType)eps->problem;
  return 0;
}
// EPSIsHermitian / EPSIsGeneralized / EPSIsPositive (epsbasic.c): from the problem type
extern "C" PetscErrorCode EPSIsHermitian(EPS eps, PetscBool *is) {
  KSG_CHECK(eps && is, PETSC_ERR_ARG_NULL, "Null argument");
  *is = ksg_eps_hermitian(eps) ? PETSC_TRUE : PETSC_FALSE;
  return 0;
}
extern "C" PetscErrorCode EPSIsGeneralized(EPS eps, PetscBool *is) {
  KSG_CHECK(eps && is, PETSC_ERR_ARG_NULL, "Null argument");
  *is = (eps->problem == EPS_GHEP || eps->problem == EPS_GNHEP) ? PETSC_TRUE : PETSC_FALSE;
  return 0;
}
extern "C" PetscErrorCode EPSIsPositive(EPS eps, PetscBool *is) {
  KSG_CHECK(eps && is, PETSC_ERR_ARG_NULL, "Null argument");
  *is = eps->problem == EPS_GHEP ? PETSC_TRUE : PETSC_FALSE;  // B positive definite (PGNHEP is not provided)
  return 0;
}

// EPSSetConvergenceTest (epsopts.c:682-700)
extern "C" PetscErrorCode EPSSetConvergenceTest(EPS eps, EPSConv conv) {
  KSG_CHECK(eps, PETSC_ERR_ARG_NULL, "Null EPS");
  KSG_CHECK(conv != EPS_CONV_USER, PETSC_ERR_SUP, "EPS_CONV_USER (a convergence test function) is not provided");
  KSG_CHECK(conv == EPS_CONV_ABS || conv == EPS_CONV_REL || conv == EPS_CONV_NORM, PETSC_ERR_ARG_OUTOFRANGE,
            "Invalid 'conv' value");
  eps->conv = conv;
  eps->setup = 0;
  return 0;
}
extern "C" PetscErrorCode EPSGetConvergenceTest(EPS eps, EPSConv *conv) {
  KSG_CHECK(eps && conv, PETSC_ERR_ARG_NULL, "Null argument");
  *conv = (EPSConv)eps->conv;
  return 0;
}
extern "C" PetscErrorCode EPSSetPurify(EPS eps, PetscBool purify) {
  KSG_CHECK(eps, PETSC_ERR_ARG_NULL, "Null EPS");
  eps->purify = purify ? 1 : 0;
  eps->setup = 0;
  return 0;
}
extern "C" PetscErrorCode EPSGetPurify(EPS eps, PetscBool *purify) {
  KSG_CHECK(eps && purify, PETSC_ERR_ARG_NULL, "Null argument");
  *purify = eps->purify ? PETSC_TRUE : PETSC_FALSE;
  return 0;
}
extern "C" PetscErrorCode EPSSetExtraction(EPS eps, EPSExtraction extr) {
  KSG_CHECK(eps, PETSC_ERR_ARG_NULL, "Null EPS");
  // EPSSetUp_KrylovSchur (krylovschur.c:120) admits Ritz and harmonic extraction
  KSG_CHECK(extr == EPS_RITZ || extr == EPS_HARMONIC, PETSC_ERR_SUP, "Unsupported extraction type");
  eps->extraction = extr;
  eps->setup = 0;
  eps->solved = 0;
  return 0;
}
extern "C" PetscErrorCode EPSGetExtraction(EPS eps, EPSExtraction *extr) {
  KSG_CHECK(eps && extr, PETSC_ERR_ARG_NULL, "Null argument");
  *extr = (EPSExtraction)eps->extraction;
  return 0;
}
extern "C" PetscErrorCode EPSSetTarget(EPS eps, PetscScalar target) {
  KSG_CHECK(eps, PETSC_ERR_ARG_NULL, "Null EPS");
  KSG_CHECK(std::isfinite(target), PETSC_ERR_ARG_WRONG, "The target must be finite");
  eps->target = target;
  eps->solved = 0;
  return 0;
}
extern "C" PetscErrorCode EPSGetTarget(EPS eps, PetscScalar *target) {
  KSG_CHECK(eps && target, PETSC_ERR_ARG_NULL, "Null argument");
  *target = eps->target;
  return 0;
}
extern "C" PetscErrorCode EPSSetDimensions(EPS eps, PetscInt nev, PetscInt ncv, PetscInt mpd) {
  KSG_CHECK(eps, PETSC_ERR_ARG_NULL, "Null EPS");
  if (nev != PETSC_CURRENT) {
    KSG_CHECK(nev > 0, PETSC_ERR_ARG_OUTOFRANGE, "Illegal value of nev. Must be > 0");
    eps->nev = nev;
  }
  if (ncv == PETSC_DETERMINE) eps->ncv = PETSC_DETERMINE;
  else if (ncv != PETSC_CURRENT) {
    KSG_CHECK(ncv > 0, PETSC_ERR_ARG_OUTOFRANGE, "Illegal value of ncv. Must be > 0");
    eps->ncv = ncv;
  }
  if (mpd == PETSC_DETERMINE) eps->mpd = PETSC_DETERMINE;
  else if (mpd != PETSC_CURRENT) {
    KSG_CHECK(mpd > 0, PETSC_ERR_ARG_OUTOFRANGE, "Illegal value of mpd. Must be > 0");
    eps->mpd = mpd;
  }
  eps->setup = 0;
  eps->solved = 0;
  return 0;
}
extern "C" PetscErrorCode EPSGetDimensions(EPS eps, PetscInt *nev, PetscInt *ncv, PetscInt *mpd) {
  KSG_CHECK(eps, PETSC_ERR_ARG_NULL, "Null EPS");
  if (nev) *nev = eps->setup ? eps->nev_e : eps->nev;
  if (ncv) *ncv = eps->setup ? eps->ncv_e : eps->ncv;
  if (mpd) *mpd = eps->setup ? eps->mpd_e : eps->mpd;
  return 0;
}
extern "C" PetscErrorCode EPSSetTolerances(EPS eps, PetscReal tol, PetscInt maxits) {
  KSG_CHECK(eps, PETSC_ERR_ARG_NULL, "Null EPS");
  if (tol == (PetscReal)PETSC_DETERMINE) eps->tol = PETSC_DETERMINE;
  else if (tol != (PetscReal)PETSC_CURRENT) {
    KSG_CHECK(tol > 0.0, PETSC_ERR_ARG_OUTOFRANGE, "Illegal value of tol. Must be > 0");
    eps->tol = tol;
  }
  if (maxits == PETSC_DETERMINE) eps->max_it = PETSC_DETERMINE;
  else if (maxits == PETSC_UNLIMITED) eps->max_it = 0x7fffffff;
  else if (maxits != PETSC_CURRENT) {
    KSG_CHECK(maxits > 0, PETSC_ERR_ARG_OUTOFRANGE, "Illegal value of maxits. Must be > 0");
    eps->max_it = maxits;
  }
  eps->setup = 0;
  eps->solved = 0;
  return 0;
}
extern "C" PetscErrorCode EPSGetTolerances(EPS eps, PetscReal *tol, PetscInt *maxits) {
  KSG_CHECK(eps, PETSC_ERR_ARG_NULL, "Null EPS");
  if (tol) *tol = eps->setup ? eps->tol_e : eps->tol;
  if (maxits) *maxits = eps->setup ? eps->maxit_e : eps->max_it;
  return 0;
}
extern "C" PetscErrorCode EPSSetWhichEigenpairs(EPS eps, EPSWhich which) {
  KSG_CHECK(eps, PETSC_ERR_ARG_NULL, "Null EPS");
  KSG_CHECK(which >= EPS_LARGEST_MAGNITUDE && which <= EPS_TARGET_REAL, PETSC_ERR_SUP,
            "Only EPS_LARGEST/SMALLEST_MAGNITUDE/REAL/IMAGINARY and EPS_TARGET_MAGNITUDE/REAL are provided "
            "(EPS_TARGET_IMAGINARY needs complex scalars)");
  eps->which = which;
  eps->solved = 0;
  return 0;
}
extern "C" PetscErrorCode EPSGetWhichEigenpairs(EPS eps, EPSWhich *which) {
  KSG_CHECK(eps && which, PETSC_ERR_ARG_NULL, "Null argument");
  *which = (EPSWhich)(eps->which ? eps->which : EPS_LARGEST_MAGNITUDE);
  return 0;
}
// EPSSetInitialSpace (epssetup.c:592-602, consumed at :400-406): the reference inserts the n vectors into the basis
// (at most ncv of them), and Krylov-Schur's factorisation starts from the first (EPSGetStartVector(eps, 0)), so the
// first vector is the one kept
extern "C" PetscErrorCode EPSSetInitialSpace(EPS eps, PetscInt n, Vec is[]) {
  KSG_CHECK(eps, PETSC_ERR_ARG_NULL, "Null EPS");
  KSG_CHECK(n >= 0, PETSC_ERR_ARG_OUTOFRANGE, "Argument n cannot be negative");
  if (n == 0) eps->v0.clear();
  else {
    KSG_CHECK(is, PETSC_ERR_ARG_NULL, "Null initial space");
    for (PetscInt i = 0; i < n; ++i) KSG_CHECK(is[i], PETSC_ERR_ARG_NULL, "Null initial vector %d", (int)i);
    eps->v0.assign(is[0]->a, is[0]->a + is[0]->n);
  }
  eps->nini = (int)n;
  eps->solved = 0;
  return 0;
}
extern "C" PetscErrorCode EPSKrylovSchurSetRestart(EPS eps, PetscReal keep) {
  KSG_CHECK(eps, PETSC_ERR_ARG_NULL, "Null EPS");
  if (keep == (PetscReal)PETSC_DETERMINE || keep == (PetscReal)PETSC_DEFAULT) eps->keep = 0.5;
  else {
    KSG_CHECK(keep >= 0.1 && keep <= 0.9, PETSC_ERR_ARG_OUTOFRANGE, "The keep argument %g must be in the range [0.1,0.9]", keep);
    eps->keep = keep;
  }
  return 0;
}
extern "C" PetscErrorCode EPSKrylovSchurGetRestart(EPS eps, PetscReal *keep) {
  KSG_CHECK(eps && keep, PETSC_ERR_ARG_NULL, "Null argument");
  *keep = eps->keep;
  return 0;
}
extern "C" PetscErrorCode EPSKrylovSchurSetLocking(EPS eps, PetscBool lock) {
  KSG_CHECK(eps, PETSC_ERR_ARG_NULL, "Null EPS");
  eps->lock = lock ? 1 : 0;
  return 0;
}
extern "C" PetscErrorCode EPSKrylovSchurGetLocking(EPS eps, PetscBool *lock) {
  KSG_CHECK(eps && lock, PETSC_ERR_ARG_NULL, "Null argument");
  *lock = eps->lock ? PETSC_TRUE : PETSC_FALSE;
  return 0;
}
extern "C" PetscErrorCode EPSGB300SetArithmetic(EPS eps, EPSGB300Arith arith) {
  KSG_CHECK(eps, PETSC_ERR_ARG_NULL, "Null EPS");
  KSG_CHECK(arith == EPS_GB300_ARITH_PAIR || arith == EPS_GB300_ARITH_F64 || arith == EPS_GB300_ARITH_F32,
            PETSC_ERR_ARG_OUTOFRANGE, "Unknown arithmetic");
  KSG_CHECK(!eps->setup || eps->arith == (int)arith, PETSC_ERR_ORDER, "Set the arithmetic before EPSSetUp");
  eps->arith = arith;
  return 0;
}
extern "C" PetscErrorCode EPSGB300GetArithmetic(EPS eps, EPSGB300Arith *arith) {
  KSG_CHECK(eps && arith, PETSC_ERR_ARG_NULL, "Null argument");
  *arith = (EPSGB300Arith)eps->arith;
  return 0;
}
extern "C" PetscErrorCode EPSGB300SetProjectedSolver(EPS eps, EPSGB300DSMethod method) {
  KSG_CHECK(eps, PETSC_ERR_ARG_NULL, "Null EPS");
  KSG_CHECK(method == EPS_GB300_DS_REFINED || method == EPS_GB300_DS_QR || method == EPS_GB300_DS_AUTO,
            PETSC_ERR_ARG_OUTOFRANGE, "Unknown projected solver");
  eps->ds_method = method;
  return 0;
}
extern "C" PetscErrorCode EPSGB300GetProjectedSolver(EPS eps, EPSGB300DSMethod *method) {
  KSG_CHECK(eps && method, PETSC_ERR_ARG_NULL, "Null argument");
  *method = (EPSGB300DSMethod)eps->ds_method;
  return 0;
}
extern "C" PetscErrorCode EPSGB300SetGSMethod(EPS eps, EPSGB300GSMethod method) {
  KSG_CHECK(eps, PETSC_ERR_ARG_NULL, "Null EPS");
  KSG_CHECK(method == EPS_GB300_GS_TENSOR || method == EPS_GB300_GS_FMA || method == EPS_GB300_GS_INTEGER ||
                method == EPS_GB300_GS_AUTO,
            PETSC_ERR_ARG_OUTOFRANGE, "Unknown Gram-Schmidt method");
  eps->gs_method = method;
  return 0;
}
extern "C" PetscErrorCode EPSGB300GetGSMethod(EPS eps, EPSGB300GSMethod *method) {
  KSG_CHECK(eps && method, PETSC_ERR_ARG_NULL, "Null argument");
  *method = (EPSGB300GSMethod)eps->gs_method;
  return 0;
}
extern "C" PetscErrorCode EPSGB300SetRestartMethod(EPS eps, EPSGB300RestartMethod method) {
  KSG_CHECK(eps, PETSC_ERR_ARG_NULL, "Null EPS");
  KSG_CHECK(method >= EPS_GB300_RESTART_TENSOR && method <= EPS_GB300_RESTART_TCGEN05, PETSC_ERR_ARG_OUTOFRANGE,
            "Unknown restart method");
  eps->restart_method = method;
  return 0;
}
extern "C" PetscErrorCode EPSGB300SetGraphCapture(EPS eps, PetscInt mode) {
  KSG_CHECK(eps, PETSC_ERR_ARG_NULL, "Null EPS");
  KSG_CHECK(mode >= -1 && mode <= 1, PETSC_ERR_ARG_OUTOFRANGE, "Graph capture mode must be -1, 0 or 1");
  eps->graph_mode = (int)mode;
  return 0;
}

extern "C" PetscErrorCode EPSGB300SetTimeLimit(EPS eps, PetscReal seconds) {
  KSG_CHECK(eps, PETSC_ERR_ARG_NULL, "Null EPS");
  eps->time_limit = seconds;
  return 0;
}
extern "C" PetscErrorCode EPSGB300SetDevice(EPS eps, int device) {
  KSG_CHECK(eps, PETSC_ERR_ARG_NULL, "Null EPS");
  int count = 0;
  KSG_CUDA(cudaGetDeviceCount(&count));
  KSG_CHECK(device >= 0 && device < count, PETSC_ERR_ARG_OUTOFRANGE, "No CUDA device %d", device);
  KSG_CHECK(!eps->setup, PETSC_ERR_ORDER, "Set the device before EPSSetUp");
  eps->device = device;
  return 0;
}

// -eps_* options from the argv given to SlepcInitialize (epsopts.c:84-260, krylovschur.c:1440-1475)
// EPSSetOptionsPrefix / EPSAppendOptionsPrefix / EPSGetOptionsPrefix (epsopts.c:1320-1400): options of this EPS are
// then spelled -<prefix>eps_..., and the reports name the prefix
extern "C" PetscErrorCode EPSSetOptionsPrefix(EPS eps, const char prefix[]) {
  KSG_CHECK(eps, PETSC_ERR_ARG_NULL, "Null EPS");
  KSG_CHECK(!prefix || prefix[0] != '-', PETSC_ERR_ARG_WRONG, "Options prefix should not begin with a hyphen");
  eps->prefix = prefix ? prefix : "";
  return 0;
}
extern "C" PetscErrorCode EPSAppendOptionsPrefix(EPS eps, const char prefix[]) {
  KSG_CHECK(eps, PETSC_ERR_ARG_NULL, "Null EPS");
  KSG_CHECK(!prefix || prefix[0] != '-', PETSC_ERR_ARG_WRONG, "Options prefix should not begin with a hyphen");
  if (prefix) eps->prefix += prefix;
  return 0;
}
extern "C" PetscErrorCode EPSGetOptionsPrefix(EPS eps, const char *prefix[]) {
  KSG_CHECK(eps && prefix, PETSC_ERR_ARG_NULL, "Null argument");
  *prefix = eps->prefix.empty() ? nullptr : eps->prefix.c_str();
  return 0;
}

extern "C" PetscErrorCode EPSSetFromOptions(EPS eps) {
  KSG_CHECK(eps, PETSC_ERR_ARG_NULL, "Null EPS");
  // STSetFromOptions and DSSetFromOptions give the default types (stset.c:125, dsbasic.c:738)
  eps->stobj.typeset = 1;
  DS ds = nullptr;
  KSG_TRY(EPSGetDS(eps, &ds));
  DSType dtype = nullptr;
  KSG_TRY(DSGetType(ds, &dtype));
  if (!dtype) KSG_TRY(DSSetType(ds, DSNHEP));
  std::string unpre;
  for (int i = 1; i < g_argc; ++i) {
    const char *o = g_argv[i];
    const char *v = (i + 1 < g_argc) ? g_argv[i + 1] : nullptr;
    if (!o || o[0] != '-') continue;
    if (!eps->prefix.empty()) {  // -<prefix>name becomes -name; options without the prefix are not this EPS's
      if (strncmp(o + 1, eps->prefix.c_str(), eps->prefix.size())) continue;
      unpre = std::string("-") + (o + 1 + eps->prefix.size());
      o = unpre.c_str();
    }
    if (!strcmp(o, "-st_type") && v) {
      // the spectral transformation is the shift of 0 (STSHIFT); the others need linear solves
      KSG_CHECK(!strcmp(v, "shift"), PETSC_ERR_SUP, "ST type %s is not provided: the shift transformation only", v);
    } else if (!strcmp(o, "-st_shift") && v) {
      KSG_CHECK(atof(v) == 0.0, PETSC_ERR_SUP, "Nonzero shifts of the spectral transformation are not provided");
    } else if (!strcmp(o, "-eps_nev") && v) KSG_TRY(EPSSetDimensions(eps, atoi(v), PETSC_CURRENT, PETSC_CURRENT));
    else if (!strcmp(o, "-eps_ncv") && v) KSG_TRY(EPSSetDimensions(eps, PETSC_CURRENT, atoi(v), PETSC_CURRENT));
    else if (!strcmp(o, "-eps_mpd") && v) KSG_TRY(EPSSetDimensions(eps, PETSC_CURRENT, PETSC_CURRENT, atoi(v)));
    else if (!strcmp(o, "-eps_tol") && v) KSG_TRY(EPSSetTolerances(eps, atof(v), PETSC_CURRENT));
    else if (!strcmp(o, "-eps_max_it") && v) KSG_TRY(EPSSetTolerances(eps, PETSC_CURRENT, atoi(v)));
    else if (!strcmp(o, "-eps_balance") && v) {  // epsopts.c:132-137: the EPSBalance names in lower case
      const char *names[] = {"none", "oneside", "twoside", "user"};
      int b = -1;
      for (int k = 0; k < 4; ++k)
        if (!strcasecmp(v, names[k])) b = k;
      KSG_CHECK(b >= 0, PETSC_ERR_USER_INPUT, "Unknown balancing method %s", v);
      KSG_TRY(EPSSetBalance(eps, (EPSBalance)b, PETSC_CURRENT, PETSC_CURRENT));
    } else if (!strcmp(o, "-eps_balance_its") && v)
      KSG_TRY(EPSSetBalance(eps, (EPSBalance)eps->balance, atoi(v), PETSC_CURRENT));
    else if (!strcmp(o, "-eps_balance_cutoff") && v)
      KSG_TRY(EPSSetBalance(eps, (EPSBalance)eps->balance, PETSC_CURRENT, atof(v)));
    else if (!strcmp(o, "-eps_largest_magnitude")) KSG_TRY(EPSSetWhichEigenpairs(eps, EPS_LARGEST_MAGNITUDE));
    else if (!strcmp(o, "-eps_smallest_magnitude")) KSG_TRY(EPSSetWhichEigenpairs(eps, EPS_SMALLEST_MAGNITUDE));
    else if (!strcmp(o, "-eps_largest_real")) KSG_TRY(EPSSetWhichEigenpairs(eps, EPS_LARGEST_REAL));
    else if (!strcmp(o, "-eps_smallest_real")) KSG_TRY(EPSSetWhichEigenpairs(eps, EPS_SMALLEST_REAL));
    else if (!strcmp(o, "-eps_largest_imaginary")) KSG_TRY(EPSSetWhichEigenpairs(eps, EPS_LARGEST_IMAGINARY));
    else if (!strcmp(o, "-eps_smallest_imaginary")) KSG_TRY(EPSSetWhichEigenpairs(eps, EPS_SMALLEST_IMAGINARY));
    else if (!strcmp(o, "-eps_target_magnitude")) KSG_TRY(EPSSetWhichEigenpairs(eps, EPS_TARGET_MAGNITUDE));
    else if (!strcmp(o, "-eps_target_real")) KSG_TRY(EPSSetWhichEigenpairs(eps, EPS_TARGET_REAL));
    else if (!strcmp(o, "-eps_target") && v) {
      // epsopts.c: giving a target also selects EPS_TARGET_MAGNITUDE unless a target criterion is already set
      KSG_TRY(EPSSetTarget(eps, atof(v)));
      if (eps->which != EPS_TARGET_REAL) KSG_TRY(EPSSetWhichEigenpairs(eps, EPS_TARGET_MAGNITUDE));
    } else if (!strcmp(o, "-eps_harmonic")) KSG_TRY(EPSSetExtraction(eps, EPS_HARMONIC));
    else if (!strcmp(o, "-eps_ritz")) KSG_TRY(EPSSetExtraction(eps, EPS_RITZ));
    else if (!strcmp(o, "-eps_hermitian")) KSG_TRY(EPSSetProblemType(eps, EPS_HEP));
    else if (!strcmp(o, "-eps_non_hermitian")) KSG_TRY(EPSSetProblemType(eps, EPS_NHEP));
    else if (!strcmp(o, "-eps_gen_hermitian")) KSG_TRY(EPSSetProblemType(eps, EPS_GHEP));
    else if (!strcmp(o, "-eps_gen_non_hermitian")) KSG_TRY(EPSSetProblemType(eps, EPS_GNHEP));
    else if (!strcmp(o, "-eps_conv_abs")) KSG_TRY(EPSSetConvergenceTest(eps, EPS_CONV_ABS));
    else if (!strcmp(o, "-eps_conv_rel")) KSG_TRY(EPSSetConvergenceTest(eps, EPS_CONV_REL));
    else if (!strcmp(o, "-eps_conv_norm")) KSG_TRY(EPSSetConvergenceTest(eps, EPS_CONV_NORM));
    else if (!strcmp(o, "-eps_monitor") || !strcmp(o, "-eps_monitor_all") || !strcmp(o, "-eps_monitor_conv")) {
      const bool has_spec = v && v[0] != '-';
      KSG_TRY(ksg_eps_monitor_from_spec(eps, !strcmp(o, "-eps_monitor") ? 0 : !strcmp(o, "-eps_monitor_all") ? 1 : 2,
                                        has_spec ? v : nullptr));
    } else if (!strcmp(o, "-eps_converged_reason") || !strcmp(o, "-eps_error_absolute") ||
               !strcmp(o, "-eps_error_relative") || !strcmp(o, "-eps_error_backward") ||
               !strcmp(o, "-eps_view_values") || !strcmp(o, "-eps_view")) {
      // reports printed at the end of EPSSolve (EPSConvergedReasonViewFromOptions, EPSErrorViewFromOptions,
      // EPSValuesViewFromOptions); the value is a viewer "[ascii][:file][:format]"
      const bool has_spec = v && v[0] != '-';
      PetscViewer pv_viewer;
      PetscViewerFormat fmt;
      int ok = 0;
      KSG_TRY(ksg_viewer_from_spec(has_spec ? v : nullptr, &pv_viewer, &fmt, &ok));
      std::string file = pv_viewer->borrowed ? std::string() : std::string(pv_viewer->name);
      if (!pv_viewer->borrowed) KSG_TRY(PetscViewerDestroy(&pv_viewer));
      if (ok) {
        EPSPostView pv;
        pv.kind = !strcmp(o, "-eps_converged_reason") ? 0
                  : !strcmp(o, "-eps_view_values")    ? 2
                  : !strcmp(o, "-eps_view")           ? 3
                                                      : 1;
        pv.etype = !strcmp(o, "-eps_error_absolute") ? EPS_ERROR_ABSOLUTE
                   : !strcmp(o, "-eps_error_backward") ? EPS_ERROR_BACKWARD
                                                       : EPS_ERROR_RELATIVE;
        pv.format = fmt;
        pv.file = file;
        eps->post_views.push_back(pv);
      }
    } else if (!strcmp(o, "-eps_purify"))
      KSG_TRY(EPSSetPurify(eps, (v && (!strcmp(v, "0") || !strcmp(v, "false"))) ? PETSC_FALSE : PETSC_TRUE));
    else if (!strcmp(o, "-eps_krylovschur_restart") && v) KSG_TRY(EPSKrylovSchurSetRestart(eps, atof(v)));
    else if (!strcmp(o, "-eps_krylovschur_locking") && v) KSG_TRY(EPSKrylovSchurSetLocking(eps, atoi(v) ? PETSC_TRUE : PETSC_FALSE));
    else if (!strcmp(o, "-eps_type") && v) KSG_TRY(EPSSetType(eps, v));
    else if (!strcmp(o, "-eps_gb300_arith") && v)
      KSG_TRY(EPSGB300SetArithmetic(eps, !strcmp(v, "f64")   ? EPS_GB300_ARITH_F64
                                         : !strcmp(v, "f32") ? EPS_GB300_ARITH_F32
                                                             : EPS_GB300_ARITH_PAIR));
    else if (!strcmp(o, "-eps_gb300_restart") && v)
      KSG_TRY(EPSGB300SetRestartMethod(eps, !strcmp(v, "pair")       ? EPS_GB300_RESTART_PAIR
                                            : !strcmp(v, "mma_sync") ? EPS_GB300_RESTART_MMA_SYNC
                                            : !strcmp(v, "tcgen05")  ? EPS_GB300_RESTART_TCGEN05
                                                                     : EPS_GB300_RESTART_TENSOR));
    else if (!strcmp(o, "-eps_gb300_ds") && v)
      KSG_TRY(EPSGB300SetProjectedSolver(eps, !strcmp(v, "qr")        ? EPS_GB300_DS_QR
                                               : !strcmp(v, "refined") ? EPS_GB300_DS_REFINED
                                                                       : EPS_GB300_DS_AUTO));
    else if (!strcmp(o, "-eps_gb300_gs") && v)
      KSG_TRY(EPSGB300SetGSMethod(eps, !strcmp(v, "fma")       ? EPS_GB300_GS_FMA
                                       : !strcmp(v, "integer") ? EPS_GB300_GS_INTEGER
                                       : !strcmp(v, "tensor")  ? EPS_GB300_GS_TENSOR
                                                               : EPS_GB300_GS_AUTO));
    else if (!strcmp(o, "-eps_gb300_graphs") && v)
      KSG_TRY(EPSGB300SetGraphCapture(eps, atoi(v)));
  }
  return 0;
}

// Generalised problems A x = lambda B x with a diagonal B = D.  The reference runs Krylov-Schur on B^-1 A (STSHIFT,
// shift 0) with the B-inner product for EPS_GHEP and the Euclidean one for EPS_GNHEP (epssetup.c:321-329,
// st/impls/shift/shift.c).  Here the iteration runs on a scaled copy of A:
//   GHEP:  C = D^-1/2 A D^-1/2 (symmetric when A is), y = D^1/2 x.  B^-1 A = D^-1/2 C D^1/2, so the Krylov space
//          of C from D^1/2 v0 is D^1/2 times that of B^-1 A from v0, and the Euclidean inner product of y-vectors
//          is the B-inner product of x-vectors: the Lanczos coefficients, Ritz values and residual estimates are
//          those of the reference; eigenvectors come back as x = D^-1/2 y.
//   GNHEP: C = D^-1 A = B^-1 A itself; vectors are unchanged.
// Each entry of C is a_rc (s_r s_c) with s = D^-1/2, one rounding per product, so C is exactly symmetric when A is.
// A non-diagonal B (k_dense.cu), the operator formed once on the device and held as a CSR matrix of its nonzero
// entries: for EPS_GNHEP C = B^-1 A (P B = L U, then the n solves), whose iteration and eigenvectors are those of
// the reference's B^-1 A with a direct solve per step; for EPS_GHEP C = L^-1 A L^-T with B = L L^T (the basis holds
// y = L^T x, and x = L^-T y wherever an eigenvector leaves the solver).
static PetscErrorCode eps_setup_general_b(EPS eps) {
  const Mat A = eps->A, B = eps->B;
  const int n = A->m;
  KSG_CHECK(!B->dense, PETSC_ERR_SUP, "A non-diagonal B must be an AIJ matrix");
  KSG_CHECK(n <= general_b_max_n(), PETSC_ERR_SUP,
            "A non-diagonal B is factorised densely on the device: at most %d rows (here %d)", general_b_max_n(), n);
  KSG_TRY(ksg_mat_upload(A));
  KSG_TRY(ksg_mat_upload(B));
  const int ghep = eps->problem == EPS_GHEP;
  DBuf<double> Bd, Cd, Td;
  DBuf<int> piv, err;
  KSG_CUDA(Bd.alloc((size_t)n * n));
  KSG_CUDA(Cd.alloc((size_t)n * n));
  KSG_CUDA(err.alloc(1));
  cudaStream_t s = eps->stream;
  KSG_CUDA(cudaMemsetAsync(err.p, 0, sizeof(int), s));
  if (ghep) {
    // B = L L^T and C = L^-1 A L^-T: the iteration runs on y = L^T x with the standard inner product, the
    // B-inner product of the reference in exact arithmetic (the diagonal case's D^1/2 scaling, generalised)
    KSG_CUDA(Td.alloc((size_t)n * n));
    KSG_CUDA(launch_general_b_ghep(A->d_rp.p, A->d_ci.p, A->d_va.p, B->d_rp.p, B->d_ci.p, B->d_va.p, n, Bd.p, Cd.p,
                                   Td.p, err.p, s));
  } else {
    KSG_CUDA(piv.alloc(n));
    KSG_CUDA(launch_general_b_operator(A->d_rp.p, A->d_ci.p, A->d_va.p, B->d_rp.p, B->d_ci.p, B->d_va.p, n, Bd.p,
                                       Cd.p, piv.p, err.p, s));
  }
  std::vector<double> c((size_t)n * n);
  int herr = 0;
  KSG_CUDA(cudaMemcpyAsync(c.data(), ghep ? Td.p : Cd.p, sizeof(double) * c.size(), cudaMemcpyDeviceToHost, s));
  KSG_CUDA(cudaMemcpyAsync(&herr, err.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  KSG_CUDA(cudaStreamSynchronize(s));
  if (ghep)
    KSG_CHECK(herr == 0, PETSC_ERR_ARG_WRONG, "EPS_GHEP needs a positive definite B (pivot %d of its Cholesky "
                                              "factorisation is not positive)", herr - 1);
  else
    KSG_CHECK(herr == 0, PETSC_ERR_ARG_WRONG, "B is singular (zero pivot in column %d of its LU factorisation)",
              herr - 1);
  if (ghep) {
    eps->d_chol.p = Bd.p;  // keep L
    eps->d_chol.count = Bd.count;
    Bd.p = nullptr;
    Bd.count = 0;
  }
  Mat C = new _p_Mat();
  C->m = C->n = n;
  C->own_i.assign(1, 0);
  for (int r = 0; r < n; ++r) {
    for (int col = 0; col < n; ++col) {
      const double v = c[(size_t)r * n + col];
      if (v != 0.0) {
        C->own_j.push_back(col);
        C->own_a.push_back(v);
      }
    }
    C->own_i.push_back((int)C->own_j.size());
  }
  C->ai = C->own_i.data();
  C->aj = C->own_j.data();
  C->aa = C->own_a.data();
  C->nnz = (long long)C->own_j.size();
  eps->op = C;
  return 0;
}

static PetscErrorCode eps_setup_operator(EPS eps) {
  eps_drop_operator(eps);
  eps->bdiag.clear();
  eps->d_bdiag.release();
  eps->d_bisqrt.release();
  eps->d_chol.release();
  if (!eps->B) {
    eps->op = eps->A;
    return 0;
  }
  const Mat A = eps->A, B = eps->B;
  const int n = A->m;
  const int ghep = eps->problem == EPS_GHEP;
  KSG_CHECK(!A->dense, PETSC_ERR_SUP, "Generalised problems need an AIJ matrix A");
  std::vector<double> d(n, 0.0);
  bool diagonal = true;
  if (B->dense) {
    for (int c = 0; c < n; ++c)
      for (int r = 0; r < n; ++r) {
        const double v = B->data[r + (size_t)c * B->lda];
        if (r == c) d[r] = v;
        else diagonal = diagonal && v == 0.0;
      }
  } else {
    for (int r = 0; r < n; ++r)
      for (int p = B->ai[r]; p < B->ai[r + 1]; ++p) {
        if (B->aj[p] == r) d[r] += B->aa[p];
        else diagonal = diagonal && B->aa[p] == 0.0;
      }
  }
  if (!diagonal) return eps_setup_general_b(eps);
  std::vector<double> sc(n);
  for (int r = 0; r < n; ++r) {
    if (ghep) {
      KSG_CHECK(d[r] > 0.0, PETSC_ERR_ARG_WRONG, "EPS_GHEP needs a positive definite B (B(%d,%d) = %g)", r, r, d[r]);
      sc[r] = 1.0 / sqrt(d[r]);
    } else {
      KSG_CHECK(d[r] != 0.0, PETSC_ERR_ARG_WRONG, "B is singular (B(%d,%d) = 0)", r, r);
      sc[r] = 1.0 / d[r];
    }
  }
  Mat C = new _p_Mat();
  C->m = C->n = n;
  C->own_i.assign(A->ai, A->ai + n + 1);
  C->own_j.assign(A->aj, A->aj + A->nnz);
  C->own_a.resize(A->nnz);
  for (int r = 0; r < n; ++r)
    for (int p = A->ai[r]; p < A->ai[r + 1]; ++p)
      C->own_a[p] = ghep ? A->aa[p] * (sc[r] * sc[A->aj[p]]) : A->aa[p] * sc[r];
  C->ai = C->own_i.data();
  C->aj = C->own_j.data();
  C->aa = C->own_a.data();
  C->nnz = A->nnz;
  eps->op = C;
  eps->bdiag.swap(d);
  KSG_CUDA(eps->d_bdiag.alloc(n));
  KSG_CUDA(cudaMemcpy(eps->d_bdiag.p, eps->bdiag.data(), sizeof(double) * n, cudaMemcpyHostToDevice));
  if (ghep) {
    KSG_CUDA(eps->d_bisqrt.alloc(n));
    KSG_CUDA(cudaMemcpy(eps->d_bisqrt.p, sc.data(), sizeof(double) * n, cudaMemcpyHostToDevice));
  }
  return 0;
}

// EPSSetUp (epssetup.c:286-418 with EPSSetUp_KrylovSchur, krylovschur.c:93-194)
extern "C" PetscErrorCode EPSSetUp(EPS eps) {
  KSG_CHECK(eps, PETSC_ERR_ARG_NULL, "Null EPS");
  if (eps->setup) {
    // set up again when an operator's values changed since (the object-state check of STSetUp)
    if (eps->A->state == eps->a_state && (!eps->B || eps->B->state == eps->b_state)) return 0;
    eps->setup = 0;
  }
  auto t0 = std::chrono::steady_clock::now();
  KSG_CHECK(eps->A, PETSC_ERR_ORDER, "EPSSetOperators must be called first");
  // the problem type against the number of matrices (epssetup.c:321-329)
  if (!eps->problem) eps->problem = eps->B ? EPS_GNHEP : EPS_NHEP;
  else if (!eps->B && (eps->problem == EPS_GHEP || eps->problem == EPS_GNHEP))
    eps->problem = (eps->problem == EPS_GHEP) ? EPS_HEP : EPS_NHEP;  // generalised without B: standard problem
  KSG_CHECK(eps->problem == EPS_HEP || eps->problem == EPS_NHEP || eps->problem == EPS_GHEP ||
                eps->problem == EPS_GNHEP, PETSC_ERR_SUP, "Unsupported problem type");
  KSG_CHECK(!eps->B || eps->problem == EPS_GHEP || eps->problem == EPS_GNHEP, PETSC_ERR_ARG_INCOMP,
            "Inconsistent EPS state: the problem type does not match the number of matrices");
  KSG_CHECK(!eps->B || eps->arith != ARITH_F32, PETSC_ERR_SUP,
            "The precision form (EPS_GB300_ARITH_F32) is provided for standard problems only");
  KSG_CHECK(ksg_eps_hermitian(eps) || (eps->balance != EPS_BALANCE_ONESIDE && eps->balance != EPS_BALANCE_TWOSIDE),
            PETSC_ERR_SUP, "Balancing of a non-Hermitian problem is not provided");
  const int n = eps->A->m;
  KSG_CHECK(n > 0, PETSC_ERR_ARG_WRONG, "Empty operator");
  int nev = eps->nev, ncv = eps->ncv, mpd = eps->mpd;
  // the dimensions clamped to the problem size (epssetup.c:336-337): ncv = n is a full basis, whose last
  // factorisation step orthogonalises A v_(n-1) against all n columns and ends in a breakdown with beta = 0
  if (nev > n) nev = n;
  if (ncv != PETSC_DETERMINE && ncv > n) ncv = n;
  // EPSSetDimensions_Default (epssetup.c:648-671)
  if (ncv != PETSC_DETERMINE) {
    KSG_CHECK(ncv >= nev + 1 || (ncv == nev && ncv == n), PETSC_ERR_USER_INPUT, "The value of ncv must be at least nev+1");
  } else if (mpd != PETSC_DETERMINE) {
    ncv = std::min(n, nev + mpd);
  } else {
    if (nev < 500) ncv = std::min(n, std::max(2 * nev, nev + 15));
    else {
      mpd = 500;
      ncv = std::min(n, nev + mpd);
    }
  }
  if (mpd == PETSC_DETERMINE) mpd = ncv;
  KSG_CHECK(ncv <= nev + mpd, PETSC_ERR_USER_INPUT, "The value of ncv must not be larger than nev+mpd");
  // projected problems: shared memory to ld = 144, then in place in the EPS's own arrays (the symmetric solver to
  // ld = 1024, the non-symmetric one to 640)
  {
    const int dsmax = ksg_eps_lanczos(eps) ? ds_hep_max_n() : ds_nhep_max_n();
    KSG_CHECK(ncv + 1 <= dsmax, PETSC_ERR_SUP,
              "ncv (%d) above %d is not provided by the device projected solver of this problem type", ncv, dsmax - 1);
  }
  KSG_CHECK(eps->lock || mpd >= ncv, PETSC_ERR_SUP, "Should not use mpd parameter in non-locking variant");
  KSG_CHECK(eps->v0.empty() || (int)eps->v0.size() == n, PETSC_ERR_ARG_SIZ, "Initial vector has the wrong length");
  // deflation spaces: the constraint columns join every projection; the harmonic, generalised and precision forms
  // keep their own bases and do not take them
  KSG_CHECK(eps->ndefl == 0 || (int)eps->defl.size() == eps->ndefl * n, PETSC_ERR_ARG_SIZ,
            "The deflation vectors have the wrong length");
  KSG_CHECK(eps->ndefl == 0 || (!eps->B && eps->extraction != EPS_HARMONIC && eps->arith != ARITH_F32),
            PETSC_ERR_SUP, "Deflation spaces are provided for standard problems with Ritz extraction in the pair or "
                           "FP64 arithmetic");
  KSG_CHECK(ncv + 1 + eps->ndefl <= gs_wide_max_columns(), PETSC_ERR_SUP,
            "ncv (%d) plus the deflation space (%d) exceeds %d columns", ncv, eps->ndefl, gs_wide_max_columns() - 1);
  KSG_CHECK(eps->nini <= ncv, PETSC_ERR_USER_INPUT, "The number of initial vectors is larger than ncv");
  eps->nev_e = nev;
  eps->ncv_e = ncv;
  eps->mpd_e = mpd;
  eps->maxit_e = (eps->max_it == PETSC_DETERMINE) ? std::max(100, 2 * n / ncv) : eps->max_it;
  eps->tol_e = (eps->tol == (double)PETSC_DETERMINE) ? 1e-8 : eps->tol;
  if (!eps->which) eps->which = EPS_LARGEST_MAGNITUDE;
  KSG_CHECK(eps->extraction == EPS_RITZ || eps->extraction == EPS_HARMONIC, PETSC_ERR_SUP, "Unsupported extraction type");
  eps->n = n;
  eps->ld = ncv + 1;
  // the device basis: columns 512-byte aligned
  eps->ldv = ((long long)n + 63) / 64 * 64;
  KSG_CUDA(cudaSetDevice(eps->device));
  if (!eps->stream) KSG_CUDA(cudaStreamCreateWithFlags(&eps->stream, cudaStreamNonBlocking));
  eps_clear_graphs(eps);  // captured segments hold the old buffers' addresses
  const int ld = eps->ld;
  eps->nc = 0;
  KSG_CUDA(eps->V.alloc((size_t)eps->ldv * (ld + 1 + eps->ndefl)));  // constraint columns, then the basis
  KSG_CUDA(cudaMemsetAsync(eps->V.p, 0, sizeof(double) * eps->V.count, eps->stream));
  KSG_CUDA(eps->d.alloc(ld + 1));
  KSG_CUDA(eps->e.alloc(ld + 1));
  KSG_CUDA(eps->H.alloc((size_t)(ld + 1) * (ld + 1)));
  KSG_CUDA(eps->Q.alloc((size_t)ld * ld));
  KSG_CUDA(eps->X.alloc((size_t)ld * ld));
  KSG_CUDA(eps->eigr.alloc(ld));
  KSG_CUDA(eps->eigi.alloc(ld));
  KSG_CUDA(eps->errest.alloc(ld));
  KSG_CUDA(eps->coef.alloc(2 * (ld + eps->ndefl) + 8));
  KSG_CUDA(eps->work.alloc(4 * ld + 8));
  KSG_CUDA(eps->dsf.alloc(ds_fast_scratch_doubles(ld)));
  KSG_CUDA(eps->rtc.alloc(restart_tc_scratch_bytes(ld)));  // grown on the first tcgen05 restart
  eps->pstride = (int)ksg_part_stride(ld + eps->ndefl);
  KSG_CUDA(eps->part.alloc(ksg_part_blocks(n) * eps->pstride));
  KSG_CUDA(eps->st.alloc(1));
  KSG_CUDA(eps->ctl.alloc(1));
  KSG_CUDA(cudaMemsetAsync(eps->st.p, 0, sizeof(KrylovState), eps->stream));
  KSG_CUDA(cudaMemsetAsync(eps->H.p, 0, sizeof(double) * eps->H.count, eps->stream));
  KSG_CUDA(cudaMemsetAsync(eps->d.p, 0, sizeof(double) * eps->d.count, eps->stream));
  KSG_CUDA(cudaMemsetAsync(eps->e.p, 0, sizeof(double) * eps->e.count, eps->stream));
  if (!eps->h_ctl) KSG_CUDA(cudaMallocHost((void **)&eps->h_ctl, sizeof(KSControl)));
  eps->storage = (eps->arith == ARITH_F64) ? STORE_F64 : STORE_PAIR;  // the precision form switches per phase
  if (eps->storage == STORE_F64) {
    // tensor-core Gram-Schmidt: the exponent table (every entry 1 until written: |v| < 2 holds for unit columns),
    // the per-block partials and the error flag
    const int ldt = ((n + 127) / 128 + 7) / 8 * 8;
    KSG_CUDA(eps->vexp.alloc((size_t)ldt * (ld + 1)));
    KSG_CUDA(cudaMemsetAsync(eps->vexp.p, 1, eps->vexp.count, eps->stream));
    KSG_CUDA(eps->gtpart.alloc(gs_tc_part_doubles()));
    KSG_CUDA(eps->gterr.alloc(1));
    KSG_CUDA(cudaMemsetAsync(eps->gterr.p, 0, sizeof(int), eps->stream));
    eps->gt.vexp = eps->vexp.p;
    eps->gt.ldt = ldt;
    eps->gt.part = eps->gtpart.p;
    eps->gt.err = eps->gterr.p;
  }
  KSG_TRY(eps_setup_operator(eps));
  Mat op = eps->op;
  KSG_TRY(ksg_mat_upload(op));
  if (op->n_seg > 0) KSG_CUDA(eps->seg_part.alloc(op->n_seg));
  if (eps->storage == STORE_PAIR) KSG_TRY(ksg_mat_upload_pairs(op));
  if (eps->arith == ARITH_F32) KSG_TRY(ksg_mat_upload_f32(op));
  // power-of-two operator scaling keeps every vector inside the range of the FP32-pair arithmetic; it is exact
  const double nrm = ksg_mat_norm_inf(op);
  eps->opscale = 1.0;
  if (nrm > 0.0 && (nrm > 1048576.0 || nrm < 1.0 / 1048576.0)) eps->opscale = ldexp(1.0, -ilogb(nrm));
  eps->lanes = spmv_lanes_for((double)op->nnz / n);
  // BVInsertConstraints: each deflation vector orthonormalised against the ones kept before it (the same two-pass
  // Gram-Schmidt kernels), a linearly dependent one dropped
  for (int i = 0; i < eps->ndefl; ++i) {
    KSG_TRY(ksg_put_column(ksg_col(eps->V.p, eps->ldv, eps->nc, eps->storage), eps->defl.data() + (size_t)i * n, n,
                           eps->storage, eps->stream));
    double cn = 0.0;
    int dep = 0;
    KSG_TRY(ksg_orthonormalize_column(eps->V.p, eps->ldv, n, eps->nc, eps->coef.p, eps->part.p, eps->pstride,
                                      eps->st.p, eps->arith, eps->stream, &cn, &dep, 2, eps->storage, nullptr));
    if (!dep && cn != 0.0) eps->nc++;
  }
  // matrix norms of EPS_CONV_NORM (epssetup.c:343-353): ||B|| only for generalised problems, else 0
  if (eps->conv == EPS_CONV_NORM) {
    eps->nrma = ksg_mat_norm_inf(eps->A);
    eps->nrmb = eps->B ? ksg_mat_norm_inf(eps->B) : 0.0;
  }
  KSG_CUDA(cudaStreamSynchronize(eps->stream));
  eps->a_state = eps->A->state;
  eps->b_state = eps->B ? eps->B->state : -1;
  // the ST and the DS the caller can query get their types here (EPSSetUp_KrylovSchur: DSHEP or DSNHEP)
  eps->stobj.typeset = 1;
  if (eps->ds) {
    KSG_TRY(DSSetType(eps->ds, ksg_eps_lanczos(eps) ? DSHEP : DSNHEP));
    if (eps->ld <= KSG_HOST_DS_MAX_LD) KSG_TRY(DSAllocate(eps->ds, eps->ld));  // the host DS is for small ld only
  }
  eps->setup = 1;
  eps->stats.setup_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  return 0;
}

// launch bracketing: counts every launch; with profiling on, records an event pair on the EPS stream
struct LaunchScope {
  EPS eps;
  int cls;
  double bytes;
  cudaEvent_t e1 = nullptr;
  LaunchScope(EPS e, int c, double b) : eps(e), cls(c), bytes(b) {
    eps->stats.kernel_launches++;
    if (eps->prof) {
      if (eps->ev_used + 2 > eps->ev_pool.size()) {
        for (int i = 0; i < 256; ++i) {
          cudaEvent_t ev;
          cudaEventCreate(&ev);
          eps->ev_pool.push_back(ev);
        }
      }
      cudaEvent_t e0 = eps->ev_pool[eps->ev_used];
      e1 = eps->ev_pool[eps->ev_used + 1];
      eps->ev_used += 2;
      cudaEventRecord(e0, eps->stream);
    }
  }
  ~LaunchScope() {
    if (eps->prof) {
      cudaEventRecord(e1, eps->stream);
      eps->ev_cls.push_back({cls, bytes});
    }
  }
};

static void prof_collect(EPS eps) {
  if (!eps->prof) return;
  for (size_t i = 0; i < eps->ev_cls.size(); ++i) {
    float ms = 0.0f;
    if (cudaEventElapsedTime(&ms, eps->ev_pool[2 * i], eps->ev_pool[2 * i + 1]) == cudaSuccess) {
      eps->prof_ms[eps->ev_cls[i].first] += ms;
      eps->prof_bytes[eps->ev_cls[i].first] += eps->ev_cls[i].second;
      eps->prof_launches[eps->ev_cls[i].first] += 1;
    }
  }
  eps->ev_cls.clear();
  eps->ev_used = 0;
}

extern "C" PetscErrorCode EPSGB300SetProfiling(EPS eps, PetscBool on) {
  KSG_CHECK(eps, PETSC_ERR_ARG_NULL, "Null EPS");
  eps->prof = on ? 1 : 0;
  for (int c = 0; c < EPS_GB300_K_COUNT; ++c) {
    eps->prof_ms[c] = 0.0;
    eps->prof_bytes[c] = 0.0;
    eps->prof_launches[c] = 0;
  }
  return 0;
}

extern "C" PetscErrorCode EPSGB300GetProfile(EPS eps, EPSGB300KernelClass cls, double *ms, double *bytes, long long *launches) {
  KSG_CHECK(eps, PETSC_ERR_ARG_NULL, "Null EPS");
  KSG_CHECK(cls >= 0 && cls < EPS_GB300_K_COUNT, PETSC_ERR_ARG_OUTOFRANGE, "Unknown kernel class");
  if (ms) *ms = eps->prof_ms[cls];
  if (bytes) *bytes = eps->prof_bytes[cls];
  if (launches) *launches = eps->prof_launches[cls];
  return 0;
}

static double spmv_bytes(EPS eps) {
  const double n = eps->n, nnz = (double)eps->op->nnz;
  return nnz * 12.0 + 4.0 * (n + 1) + 16.0 * n;
}

// one Krylov factorisation segment: steps k0..nv-1 plus the final reorthogonalisation of the residual vector
static PetscErrorCode eps_factorize_launch(EPS eps, int k0, int nv, double *bytes) {
  cudaStream_t s = eps->stream;
  const int n = eps->n;
  const int herm = ksg_eps_lanczos(eps);
  KSG_CUDA(launch_segment_begin(eps->st.p, k0, nv, s));
  StepArgs a = {};
  a.V = eps->V.p;
  a.ldv = eps->ldv;
  a.n = n;
  a.hermitian = herm;
  a.d = eps->d.p;
  a.e = eps->e.p;
  a.H = eps->H.p;
  a.ldh = eps->ld;
  a.eta = 0.7071;
  a.coef = eps->coef.p;
  a.part = eps->part.p;
  a.pstride = eps->pstride;
  a.st = eps->st.p;
  a.tc = eps->gs_tc_on ? &eps->gt : nullptr;
  a.nc = eps->nc;
  const int nc = eps->nc;
  const double colb = 8.0 * n;
  const Mat op = eps->op;
  LongRows lr;
  if (op->n_long > 0) {
    lr.n_long = op->n_long;
    lr.n_seg = op->n_seg;
    lr.long_t = LONG_ROW_T;
    lr.seg_row = op->d_seg_row.p;
    lr.seg_beg = op->d_seg_beg.p;
    lr.seg_end = op->d_seg_end.p;
    lr.lrow = op->d_lrow.p;
    lr.lfirst = op->d_lfirst.p;
    lr.part = eps->seg_part.p;
  }
  for (int j = k0; j < nv; ++j) {
    void *u = ksg_col(eps->V.p, eps->ldv, nc + j, eps->storage);
    void *w = ksg_col(eps->V.p, eps->ldv, nc + j + 1, eps->storage);
    {
      LaunchScope ls(eps, EPS_GB300_K_SPMV, spmv_bytes(eps));
      KSG_CUDA(launch_spmv_storage(op->d_rp.p, op->d_ci.p, op->d_va.p, op->d_va2.p, u, w, n, eps->lanes, eps->st.p,
                                   eps->opscale, eps->storage, s, &lr, op->d_va32.p));
    }
    a.J = nc + j;  // the constraint columns, then Krylov columns 0..j-1
    a.j = j;
    a.U = u;
    a.W = w;
    {
      LaunchScope ls(eps, EPS_GB300_K_GS_DOT, colb * (j + 2));
      KSG_CUDA(launch_gs_dot(a, 2, GS_STEP, eps->arith, s, eps->storage));
    }
    {
      LaunchScope ls(eps, EPS_GB300_K_GS_UPDATE, colb * (j + 4));
      KSG_CUDA(launch_gs_update(a, 2, GS_STEP, eps->arith, s, eps->storage));
    }
    *bytes += spmv_bytes(eps) + colb * (j + 2) + colb * (j + 4);
  }
  a.J = nc + nv;
  a.j = nv;
  a.U = ksg_col(eps->V.p, eps->ldv, nc + nv, eps->storage);
  a.W = nullptr;
  {
    LaunchScope ls(eps, EPS_GB300_K_GS_DOT, colb * (nv + 1));
    KSG_CUDA(launch_gs_dot(a, 1, GS_FINAL, eps->arith, s, eps->storage));
  }
  {
    LaunchScope ls(eps, EPS_GB300_K_GS_UPDATE, colb * (nv + 2));
    KSG_CUDA(launch_gs_update(a, 1, GS_FINAL, eps->arith, s, eps->storage));
  }
  *bytes += colb * (nv + 1) + colb * (nv + 2);
  eps->stats.kernel_launches += 1;  // segment begin
  eps->stats.krylov_steps += nv - k0;
  return 0;
}

// One factorisation segment: direct launches the first time a (k, nv) segment runs, a captured CUDA graph from the
// second time on (the same kernels with the same arguments; the stop flag in the device state ends a segment early
// in either form).  A capture that fails turns graphs off for this EPS and runs the launches directly.
static PetscErrorCode eps_factorize(EPS eps, int k0, int nv, double *bytes) {
  const bool on = eps->graph_mode == 1 || (eps->graph_mode == -1 && eps->n <= kGraphMaxRows);
  if (!on || eps->prof || eps->gs_tc_on) return eps_factorize_launch(eps, k0, nv, bytes);
  const std::array<int, 4> key = {k0, nv, eps->storage, eps->arith};
  auto it = eps->seg_graphs.find(key);
  if (it == eps->seg_graphs.end()) {
    if (eps->seg_graphs.size() >= 512) return eps_factorize_launch(eps, k0, nv, bytes);
    it = eps->seg_graphs.emplace(key, _p_EPS::SegGraph()).first;
  }
  _p_EPS::SegGraph &g = it->second;
  if (!g.exec) {
    if (++g.seen < 2) return eps_factorize_launch(eps, k0, nv, bytes);
    const long long l0 = eps->stats.kernel_launches, s0 = eps->stats.krylov_steps;
    double b = 0.0;
    cudaGraph_t graph = nullptr;
    cudaError_t ce = cudaStreamBeginCapture(eps->stream, cudaStreamCaptureModeThreadLocal);
    PetscErrorCode ierr = 0;
    if (ce == cudaSuccess) {
      ierr = eps_factorize_launch(eps, k0, nv, &b);
      ce = cudaStreamEndCapture(eps->stream, &graph);
    }
    cudaGraphExec_t exec = nullptr;
    if (!ierr && ce == cudaSuccess && graph) ce = cudaGraphInstantiate(&exec, graph, 0);
    if (graph) cudaGraphDestroy(graph);
    const long long captured = eps->stats.kernel_launches - l0;  // the kernels the capture recorded
    eps->stats.kernel_launches = l0;
    eps->stats.krylov_steps = s0;
    if (ierr || ce != cudaSuccess || !exec) {
      if (exec) cudaGraphExecDestroy(exec);
      cudaGetLastError();  // the capture's error is not the solve's: the launches run directly from here on
      eps->graph_mode = 0;
      return eps_factorize_launch(eps, k0, nv, bytes);
    }
    g.exec = exec;
    g.launches = captured;
    g.bytes = b;
  }
  KSG_CUDA(cudaGraphLaunch(g.exec, eps->stream));
  eps->stats.kernel_launches += g.launches;
  eps->stats.krylov_steps += nv - k0;
  eps->stats.graph_segments++;
  *bytes += g.bytes;
  return 0;
}

// the Krylov basis: column nc of V (the constraint columns of a deflation space come first), as a double pointer
// whose column stride is ldv 8-byte entries in the pair and FP64 formats
static inline double *eps_basis(EPS eps) {
  return static_cast<double *>(ksg_col(eps->V.p, eps->ldv, eps->nc, eps->storage));
}

// basis column <-> FP64 device vector, for the pair and FP64 storage formats
static cudaError_t eps_column_to_f64(EPS eps, int col, double *x, cudaStream_t s) {
  const void *c = ksg_col(eps->V.p, eps->ldv, eps->nc + col, eps->storage);
  if (eps->storage == STORE_PAIR) return launch_pair_to_f64(static_cast<const float2 *>(c), x, eps->n, s);
  return cudaMemcpyAsync(x, c, sizeof(double) * eps->n, cudaMemcpyDeviceToDevice, s);
}
static cudaError_t eps_f64_to_column(EPS eps, const double *x, int col, cudaStream_t s) {
  void *c = ksg_col(eps->V.p, eps->ldv, eps->nc + col, eps->storage);
  if (eps->storage == STORE_PAIR) return launch_f64_to_pair(x, static_cast<float2 *>(c), eps->n, s);
  return cudaMemcpyAsync(c, x, sizeof(double) * eps->n, cudaMemcpyDeviceToDevice, s);
}

// EPSGetStartVector's "force the vector into the range of OP" for definite generalised problems
// (epssolve.c:855-862): basis column col <- C column col, in FP64 on the device
static PetscErrorCode eps_apply_op_column(EPS eps, int col, cudaStream_t s) {
  DBuf<double> x, y;
  KSG_CUDA(x.alloc(eps->n));
  KSG_CUDA(y.alloc(eps->n));
  KSG_CUDA(eps_column_to_f64(eps, col, x.p, s));
  KSG_CUDA(launch_spmv(eps->op->d_rp.p, eps->op->d_ci.p, eps->op->d_va.p, x.p, y.p, eps->n, eps->lanes, nullptr,
                       eps->opscale, s));
  KSG_CUDA(eps_f64_to_column(eps, y.p, col, s));
  KSG_CUDA(cudaStreamSynchronize(s));  // x and y are freed on return
  eps->stats.kernel_launches += 1 + (eps->storage == STORE_PAIR ? 2 : 0);
  return 0;
}

// the initial space, or a random vector, into column 0 of the basis (not yet normalised); for EPS_GHEP the user's
// vector v0 becomes D^1/2 v0 (the basis holds y = D^1/2 x) and is then mapped into the range of the operator
PetscErrorCode ksg_eps_put_start(EPS eps, cudaStream_t s) {
  std::vector<double> h;
  const double *src;
  if (!eps->v0_internal.empty()) src = eps->v0_internal.data();  // the precision form's refinement sweep
  else if (!eps->v0.empty()) {
    src = eps->v0.data();
    if (eps->problem == EPS_GHEP && eps->B && eps->d_chol.p) {
      // y0 = L^T v0 on the device, then into the range of the operator
      const int n = eps->n;
      DBuf<double> x, y;
      KSG_CUDA(x.alloc(n));
      KSG_CUDA(y.alloc(n));
      KSG_CUDA(cudaMemcpyAsync(x.p, eps->v0.data(), sizeof(double) * n, cudaMemcpyHostToDevice, s));
      KSG_CUDA(launch_lt_mv(eps->d_chol.p, x.p, y.p, n, s));
      KSG_CUDA(eps_f64_to_column(eps, y.p, 0, s));
      KSG_CUDA(cudaStreamSynchronize(s));
      KSG_TRY(eps_apply_op_column(eps, 0, s));
      return 0;
    }
    if (eps->problem == EPS_GHEP && eps->B) {
      h.resize(eps->n);
      for (int r = 0; r < eps->n; ++r) h[r] = eps->v0[r] * sqrt(eps->bdiag[r]);
      src = h.data();
    }
  } else {
    h.resize(eps->n);
    ksg_random_fill(h.data(), eps->n, eps->seed, 0);
    src = h.data();
  }
  KSG_TRY(ksg_put_column(ksg_col(eps->V.p, eps->ldv, eps->nc, eps->storage), src, eps->n, eps->storage, s));
  KSG_CUDA(cudaStreamSynchronize(s));  // h is pageable and goes out of scope
  if (eps->problem == EPS_GHEP && eps->B) KSG_TRY(eps_apply_op_column(eps, 0, s));
  return 0;
}

PetscErrorCode ksg_eps_new_start_vector(EPS eps, int col, int *breakdown) {
  std::vector<double> h(eps->n);
  ksg_random_fill(h.data(), eps->n, eps->seed, ++eps->rng_counter);
  void *dst = ksg_col(eps->V.p, eps->ldv, eps->nc + col, eps->storage);
  KSG_TRY(ksg_put_column(dst, h.data(), eps->n, eps->storage, eps->stream));
  if (eps->problem == EPS_GHEP && eps->B) KSG_TRY(eps_apply_op_column(eps, col, eps->stream));
  double nrm = 0.0;
  int ld = 0;
  KSG_TRY(ksg_orthonormalize_column(eps->V.p, eps->ldv, eps->n, eps->nc + col, eps->coef.p, eps->part.p,
                                    eps->pstride, eps->st.p, eps->arith, eps->stream, &nrm, &ld, 2, eps->storage,
                                    eps->gs_tc_on ? &eps->gt : nullptr));
  *breakdown = ld || nrm == 0.0;
  return 0;
}

static int compare_which(int which, double target, double ar, double ai, double br, double bi) {
  double a, b;
  switch (which) {
    case EPS_TARGET_MAGNITUDE: a = hypot(ar - target, ai); b = hypot(br - target, bi); return a > b ? 1 : (a < b ? -1 : 0);
    case EPS_TARGET_REAL: a = fabs(ar - target); b = fabs(br - target); return a > b ? 1 : (a < b ? -1 : 0);
    case EPS_LARGEST_MAGNITUDE: a = hypot(ar, ai); b = hypot(br, bi); return a < b ? 1 : (a > b ? -1 : 0);
    case EPS_SMALLEST_MAGNITUDE: a = hypot(ar, ai); b = hypot(br, bi); return a > b ? 1 : (a < b ? -1 : 0);
    case EPS_LARGEST_REAL: return ar < br ? 1 : (ar > br ? -1 : 0);
    case EPS_SMALLEST_REAL: return ar > br ? 1 : (ar < br ? -1 : 0);
    case EPS_LARGEST_IMAGINARY: a = fabs(ai); b = fabs(bi); return a < b ? 1 : (a > b ? -1 : 0);
    case EPS_SMALLEST_IMAGINARY: a = fabs(ai); b = fabs(bi); return a > b ? 1 : (a < b ? -1 : 0);
  }
  return 0;
}

// SlepcSortEigenvalues (slepcsc.c:89-140): insertion sort keeping conjugate pairs together
static void sort_eigenvalues(int which, double target, int n, const double *eigr, const double *eigi, int *perm) {
  for (int i = n - 1; i >= 0; i--) {
    double re = eigr[perm[i]], im = eigi[perm[i]];
    int j = i + 1;
    if (im != 0.0) {
      i--;
      im = eigi[perm[i]];
    }
    while (j < n) {
      if (compare_which(which, target, re, im, eigr[perm[j]], eigi[perm[j]]) <= 0) break;
      int tmp;
      if (im == 0.0) {
        if (eigi[perm[j]] == 0.0) {
          tmp = perm[j - 1]; perm[j - 1] = perm[j]; perm[j] = tmp; j++;
        } else {
          tmp = perm[j - 1]; perm[j - 1] = perm[j]; perm[j] = perm[j + 1]; perm[j + 1] = tmp; j += 2;
        }
      } else {
        if (eigi[perm[j]] == 0.0) {
          tmp = perm[j - 2]; perm[j - 2] = perm[j]; perm[j] = perm[j - 1]; perm[j - 1] = tmp; j++;
        } else {
          tmp = perm[j - 2]; perm[j - 2] = perm[j]; perm[j] = tmp;
          tmp = perm[j - 1]; perm[j - 1] = perm[j + 1]; perm[j + 1] = tmp; j += 2;
        }
      }
    }
  }
}

// EPSSolve (epssolve.c:119-208) with EPSSolve_KrylovSchur_Default (krylovschur.c:227-337) on the device
// undo the operator scaling and order the results (epssolve.c:159-178); eigr/eigi/errest are the device arrays
// already copied to the host; conjugate pairs with a negative first imaginary part are flipped on the device
PetscErrorCode ksg_eps_assemble(EPS eps, int nconv, const double *er, const double *ei, const double *es,
                                cudaStream_t s) {
  const int n = eps->n;
  const int herm = ksg_eps_hermitian(eps);
  eps->r_eigr.assign(er, er + nconv);
  eps->r_eigi.assign(ei, ei + nconv);
  eps->r_errest.assign(es, es + nconv);
  if (herm) std::fill(eps->r_eigi.begin(), eps->r_eigi.end(), 0.0);
  for (int i = 0; i < nconv; ++i) {
    eps->r_eigr[i] /= eps->opscale;
    eps->r_eigi[i] /= eps->opscale;
  }
  for (int i = 0; i < nconv - 1; ++i) {
    if (eps->r_eigi[i] != 0.0) {
      if (eps->r_eigi[i] < 0.0) {
        eps->r_eigi[i] = -eps->r_eigi[i];
        eps->r_eigi[i + 1] = -eps->r_eigi[i + 1];
        // negate a basis column: both halves of a pair, the float, or the double
        KSG_CUDA(launch_negate(ksg_col(eps->V.p, eps->ldv, eps->nc + i + 1, eps->storage),
                               eps->storage == STORE_PAIR ? 2 * n : n, eps->storage != STORE_F64, s));
      }
      i++;
    }
  }
  eps->perm.resize(std::max(nconv, 1));
  for (int i = 0; i < nconv; ++i) eps->perm[i] = i;
  sort_eigenvalues(eps->which, eps->target, nconv, eps->r_eigr.data(), eps->r_eigi.data(), eps->perm.data());
  return 0;
}

// V(:, s0:s0+N) = V(:, a0:a0+K) Q(a0:a0+K, s0:s0+N): the tensor-core restart for pair storage and (tcgen05) for FP64
// storage, the CUDA-core kernel of the storage's arithmetic otherwise
// the tensor-core kernel of EPS_GB300_RESTART_TENSOR: tcgen05 (bit-identical to mma.sync; the 128^3 Laplacian's
// restarts take 417 ms per solve against 782 ms)
static const bool kRestartTensorIsTcgen05 = true;

static cudaError_t eps_restart(EPS eps, int a0, int K, int s0, int N, const double *Q, cudaStream_t s) {
  const int m = eps->restart_method;
  const bool t5 = m == EPS_GB300_RESTART_TCGEN05 || (m == EPS_GB300_RESTART_TENSOR && kRestartTensorIsTcgen05);
  // the tensor-core restarts stage up to 144 columns of Q; wider bases take the CUDA-core kernel
  const bool narrow = eps->ld <= 144;
  if (narrow && ((eps->storage == STORE_PAIR && m != EPS_GB300_RESTART_PAIR) || (eps->storage == STORE_F64 && t5))) {
    if (t5) {
      const size_t need = restart_t5_scratch_bytes(eps->ld);  // about 2 KB per SM and basis column
      if (eps->rtc.count < need) {
        cudaError_t e = eps->rtc.alloc(need);
        if (e == cudaSuccess) e = cudaMemsetAsync(eps->rtc.p, 0, need, s);
        if (e != cudaSuccess) return e;
      }
      if (eps->storage == STORE_F64)
        return launch_restart_t5_f64(eps_basis(eps), eps->ldv, eps->n, a0, K, s0, N, Q, eps->ld, eps->rtc.p, eps->ld, s,
                                     eps->vexp.p, eps->gt.ldt);
      return launch_restart_t5(reinterpret_cast<float2 *>(eps_basis(eps)), eps->ldv, eps->n, a0, K, s0, N, Q, eps->ld,
                               eps->rtc.p, eps->ld, s);
    }
    return launch_restart_tc(reinterpret_cast<float2 *>(eps_basis(eps)), eps->ldv, eps->n, a0, K, s0, N, Q, eps->ld,
                             eps->rtc.p, eps->ld, s);
  }
  return launch_restart(eps_basis(eps), eps->ldv, eps->n, a0, K, s0, N, Q, eps->ld, eps->arith, s, eps->storage);
}

__global__ void k_residual(const double *y, const double *yi, const double *x, const double *xi, const double *b,
                           double kr, double ki, int n, double *part);

// EPS_Purify + BVNormalize for EPS_GHEP (epsdefault.c:28-50, epsimpl.h:297-312): x <- B^-1 A x, B-normalised.  In
// the basis y = D^1/2 x this is y <- C y / ||C y||, on the device for the first m columns.
static PetscErrorCode eps_purify(EPS eps, int m, cudaStream_t s, double *bytes) {
  const int n = eps->n;
  const int blocks = std::min(1024, (n + 255) / 256);
  DBuf<double> x, y, part;
  KSG_CUDA(x.alloc(n));
  KSG_CUDA(y.alloc(n));
  KSG_CUDA(part.alloc(3 * blocks));
  std::vector<double> h(3 * blocks);
  for (int j = 0; j < m; ++j) {
    KSG_CUDA(eps_column_to_f64(eps, j, x.p, s));
    KSG_CUDA(launch_spmv(eps->op->d_rp.p, eps->op->d_ci.p, eps->op->d_va.p, x.p, y.p, n, eps->lanes, nullptr, 1.0,
                         s));
    k_residual<<<blocks, 256, 0, s>>>(y.p, nullptr, y.p, nullptr, nullptr, 0.0, 0.0, n, part.p);
    KSG_CUDA(cudaGetLastError());
    KSG_CUDA(cudaMemcpyAsync(h.data(), part.p, sizeof(double) * 3 * blocks, cudaMemcpyDeviceToHost, s));
    KSG_CUDA(cudaStreamSynchronize(s));
    double ss = 0.0;
    for (int b = 0; b < blocks; ++b) ss += h[3 * b];
    KSG_CHECK(ss > 0.0, PETSC_ERR_PLIB, "Purification gave a zero vector (column %d)", j);
    KSG_CUDA(launch_scale(y.p, n, 1.0 / sqrt(ss), s));
    KSG_CUDA(eps_f64_to_column(eps, y.p, j, s));
    eps->stats.kernel_launches += 4 + (eps->storage == STORE_PAIR ? 2 : 0);
    *bytes += 8.0 * n * 8 + spmv_bytes(eps);
  }
  KSG_CUDA(cudaStreamSynchronize(s));
  return 0;
}

// One Krylov-Schur solve in the current storage format with tolerance tol (the body of EPSSolve): start vector,
// restart loop, eigenvectors of the Schur form, results assembled into the EPS.
static PetscErrorCode eps_solve_core(EPS eps, double tol, std::chrono::steady_clock::time_point t0, int *nconv_out,
                                     int *its_out, int *reason_out, double *bytes_out) {
  cudaStream_t s = eps->stream;
  const int n = eps->n, ld = eps->ld, ncv = eps->ncv_e, mpd = eps->mpd_e, nev = eps->nev_e;
  const int herm = ksg_eps_lanczos(eps);
  const int harmonic = eps->extraction == EPS_HARMONIC;
  // IEEE-double Gram-Schmidt with exact products (tensor cores or integer pipes): the symmetric (Lanczos) variant
  // with the tcgen05 restart, whose kernels and these keep the basis columns' exponent table up to date
  {
    const int rm = eps->restart_method;
    // the automatic choice: exact integer products unless the segments will replay from CUDA graphs
    const bool graphs = eps->graph_mode == 1 || (eps->graph_mode == -1 && n <= kGraphMaxRows);
    const int exact = eps->gs_method == EPS_GB300_GS_TENSOR || eps->gs_method == EPS_GB300_GS_INTEGER ||
                      (eps->gs_method == EPS_GB300_GS_AUTO && !graphs);
    eps->gs_tc_on = eps->storage == STORE_F64 && eps->arith == ARITH_F64 && exact && herm && eps->vexp.p &&
                    ld <= gs_tc_max_columns() && ncv < n && eps->nc == 0 &&
                    (rm == EPS_GB300_RESTART_TCGEN05 || (rm == EPS_GB300_RESTART_TENSOR && kRestartTensorIsTcgen05));
    eps->gt.integer = eps->gs_method != EPS_GB300_GS_TENSOR;
    if (eps->gs_tc_on) eps->stats.gs_exact = 1;
    if (eps->gs_tc_on) KSG_CUDA(cudaMemsetAsync(eps->gterr.p, 0, sizeof(int), s));
  }
  // start vector: the initial space, or a random vector (EPSGetStartVector, epssolve.c:841-873)
  {
    KSG_TRY(ksg_eps_put_start(eps, s));
    double nrm = 0.0;
    int lindep = 0;
    // against the constraint columns (if any) with refinement as needed, else a normalisation
    KSG_TRY(ksg_orthonormalize_column(eps->V.p, eps->ldv, n, eps->nc, eps->coef.p, eps->part.p, eps->pstride,
                                      eps->st.p, eps->arith, s, &nrm, &lindep, eps->nc ? 0 : 1, eps->storage,
                                      eps->gs_tc_on ? &eps->gt : nullptr));
    KSG_CHECK(!lindep && nrm != 0.0, PETSC_ERR_PLIB, "Initial vector is zero or belongs to the deflation space");
  }
  KSG_CUDA(cudaMemsetAsync(eps->d.p, 0, sizeof(double) * eps->d.count, s));
  KSG_CUDA(cudaMemsetAsync(eps->e.p, 0, sizeof(double) * eps->e.count, s));
  KSG_CUDA(cudaMemsetAsync(eps->H.p, 0, sizeof(double) * eps->H.count, s));
  int nconv = 0, l = 0, its = 0, reason = 0;
  double bytes = 0.0;
  // the mixed-precision projected solver while it passes its checks (EPS_GB300_DS_AUTO: until a restart falls back
  // to the QR solver, whose result that restart then uses)
  bool ds_refined =
      herm && ld <= 144 && (eps->ds_method == EPS_GB300_DS_REFINED || eps->ds_method == EPS_GB300_DS_AUTO);
  int ds_fb_run = 0;
  while (reason == 0) {
    its++;
    int nv = std::min(nconv + mpd, ncv);
    const int k0 = nconv + l;
    KSG_CHECK(nv > k0, PETSC_ERR_PLIB, "Internal error: empty Krylov segment (nv=%d, k=%d)", nv, k0);
    KSG_TRY(eps_factorize(eps, k0, nv, &bytes));
    DSArgs da = {};
    da.ld = ld;
    da.n = nv;
    da.flags = DS_DO_ALL;
    da.l = nconv;
    da.k = k0;
    da.raw = l > 0;
    da.d = eps->d.p;
    da.e = eps->e.p;
    da.H = eps->H.p;
    da.Q = eps->Q.p;
    da.eigr = eps->eigr.p;
    da.eigi = eps->eigi.p;
    da.errest = eps->errest.p;
    da.work = eps->work.p;
    da.which = eps->which;
    da.tol = tol;
    da.nev = nev;
    da.its = its;
    da.max_it = eps->maxit_e;
    da.keep = eps->keep;
    da.lock = eps->lock;
    da.st = eps->st.p;
    da.ctl = eps->ctl.p;
    da.target = eps->target * eps->opscale;  // the projected problem holds the scaled operator
    da.harmonic = harmonic;
    da.conv = eps->conv == EPS_CONV_ABS ? DS_CONV_ABS : eps->conv == EPS_CONV_NORM ? DS_CONV_NORM : DS_CONV_REL;
    da.conv_a = eps->conv == EPS_CONV_NORM ? eps->nrma * eps->opscale : eps->opscale;
    da.conv_b = eps->nrmb;
    {
      LaunchScope ls(eps, EPS_GB300_K_DS, 0.0);
      if (ds_refined) {
        KSG_CUDA(launch_ds_hep_fast(da, ds_fast_layout(eps->dsf.p, ld), ld, s));
        eps->stats.kernel_launches += ds_fast_launches() - 1;
      } else if (herm) {
        KSG_CUDA(launch_ds_hep(da, ld, s));
      } else {
        KSG_CUDA(launch_ds_nhep(da, ld, s));
      }
    }
    KSG_CUDA(cudaMemcpyAsync(eps->h_ctl, eps->ctl.p, sizeof(KSControl), cudaMemcpyDeviceToHost, s));
    KSG_CUDA(cudaStreamSynchronize(s));
    prof_collect(eps);
    const KSControl c = *eps->h_ctl;
    KSG_CHECK(!c.ds_error, PETSC_ERR_LIB, "The projected eigenproblem solver did not converge (restart %d)", its);
    if (ds_refined) {
      if (c.ds_fallback) {
        eps->stats.ds_fallbacks++;
        if (++ds_fb_run >= 1 && eps->ds_method == EPS_GB300_DS_AUTO) ds_refined = false;
      } else {
        ds_fb_run = 0;
      }
    }
    const int k = c.nconv;
    l = c.l;
    reason = c.reason;
    nv = c.nv;
    if (!eps->mon.empty()) KSG_TRY(eps_run_monitors(eps, its, k, nv, s));
    if (harmonic && reason == 0 && !(c.breakdown || k == nv)) {
      // undo the harmonic translation on the residual vector (krylovschur.c:312-315): gamma u^ = u - V(:,0:nv) g~,
      // with g~ from the projected solver (work) and gamma in the control block; the BVMultVec form of the
      // Gram-Schmidt update kernel
      StepArgs ha = {};
      ha.V = eps_basis(eps);  // (no constraint columns with harmonic extraction)
      ha.ldv = eps->ldv;
      ha.n = n;
      ha.J = nv;
      ha.j = nv;
      ha.hermitian = 1;
      ha.U = ksg_col(eps_basis(eps), eps->ldv, nv, eps->storage);
      ha.eta = 0.7071;
      ha.coef = eps->work.p;
      ha.part = eps->part.p;
      ha.pstride = eps->pstride;
      ha.st = eps->st.p;
      KSG_CUDA(launch_set_scales(eps->st.p, 1.0, 1.0 / c.hgamma, s));
      KSG_CUDA(launch_gs_update(ha, 1, GS_COMBINE, eps->arith, s, eps->storage));
      eps->stats.kernel_launches += 2;
      bytes += 8.0 * n * (nv + 2);
    }
    // thick restart: V(:, nconv:k+l) = V(:, nconv:nv) Q(nconv:nv, nconv:k+l)
    {
      LaunchScope ls(eps, EPS_GB300_K_RESTART, 8.0 * n * ((nv - nconv) + (k + l - nconv)));
      KSG_CUDA(eps_restart(eps, nconv, nv - nconv, nconv, k + l - nconv, eps->Q.p, s));
    }
    bytes += 8.0 * n * ((nv - nconv) + (k + l - nconv));
    if (reason == 0) {
      if (c.breakdown || k == nv) {
        // start a new Krylov factorisation at column k (after the rotation of the converged vectors)
        if (k < nev) {
          int bd = 0;
          KSG_TRY(ksg_eps_new_start_vector(eps, k, &bd));
          if (bd) reason = EPS_DIVERGED_BREAKDOWN;
        }
      } else {
        KSG_CUDA(cudaMemcpyAsync(ksg_col(eps_basis(eps), eps->ldv, k + l, eps->storage),
                                 ksg_col(eps_basis(eps), eps->ldv, nv, eps->storage), ksg_entry_bytes(eps->storage) * n,
                                 cudaMemcpyDeviceToDevice, s));
      }
    }
    nconv = k;
    eps->stats.restarts++;
    if (reason == 0 && eps->time_limit > 0.0 &&
        std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count() > eps->time_limit)
      reason = EPS_DIVERGED_ITS;  // the caller's wall-time budget ran out (EPSGB300SetTimeLimit)
  }
  // non-Hermitian or harmonic: eigenvectors of the leading Schur block, V = V X (EPSComputeVectors_Schur,
  // epsdefault.c:105-169)
  if (!herm && nconv > 0) {
    KSG_CUDA(launch_nhep_vectors(eps->H.p, ld, nconv, eps->X.p, s));
    KSG_CUDA(eps_restart(eps, 0, nconv, 0, nconv, eps->X.p, s));
    bytes += 16.0 * n * nconv;
  }
  if (eps->problem == EPS_GHEP && eps->B && eps->purify && nconv > 0) KSG_TRY(eps_purify(eps, nconv, s, &bytes));
  std::vector<double> er(ld), ei(ld), es(ld);
  KSG_CUDA(cudaMemcpyAsync(er.data(), eps->eigr.p, sizeof(double) * ld, cudaMemcpyDeviceToHost, s));
  KSG_CUDA(cudaMemcpyAsync(ei.data(), eps->eigi.p, sizeof(double) * ld, cudaMemcpyDeviceToHost, s));
  KSG_CUDA(cudaMemcpyAsync(es.data(), eps->errest.p, sizeof(double) * ld, cudaMemcpyDeviceToHost, s));
  KSG_CUDA(cudaStreamSynchronize(s));
  KSG_TRY(ksg_eps_assemble(eps, nconv, er.data(), ei.data(), es.data(), s));
  *nconv_out = nconv;
  *its_out = its;
  *reason_out = reason;
  *bytes_out = bytes;
  return 0;
}

// in-place widening of basis columns [0, m) from FP32 to pairs (same leading dimension, twice the bytes); columns
// are converted from the last down (column j's pairs overwrite the floats of columns 2j and 2j+1, converted
// before it), column 0 through a temporary
PetscErrorCode ksg_eps_widen_f32(EPS eps, int m) {
  cudaStream_t s = eps->stream;
  const int n = eps->n;
  DBuf<double> tmp;
  KSG_CUDA(tmp.alloc(n));
  for (int j = m - 1; j >= 0; --j) {
    const float *src = static_cast<const float *>(ksg_col(eps->V.p, eps->ldv, j, STORE_F32));
    KSG_CUDA(launch_f32_to_f64(src, tmp.p, n, s));
    KSG_CUDA(launch_f64_to_pair(tmp.p, static_cast<float2 *>(ksg_col(eps->V.p, eps->ldv, j, STORE_PAIR)), n, s));
  }
  KSG_CUDA(cudaStreamSynchronize(s));
  return 0;
}

extern "C" PetscErrorCode EPSSolve(EPS eps) {
  KSG_CHECK(eps, PETSC_ERR_ARG_NULL, "Null EPS");
  KSG_TRY(EPSSetUp(eps));
  KSG_CUDA(cudaSetDevice(eps->device));
  cudaStream_t s = eps->stream;
  eps->xvec_valid = 0;  // the device eigenvectors of an earlier solve are stale
  auto t0 = std::chrono::steady_clock::now();
  if (!eps->ev_solve[0]) {
    KSG_CUDA(cudaEventCreate(&eps->ev_solve[0]));
    KSG_CUDA(cudaEventCreate(&eps->ev_solve[1]));
  }
  KSG_CUDA(cudaEventRecord(eps->ev_solve[0], s));
  eps->stats.krylov_steps = 0;
  eps->stats.restarts = 0;
  eps->stats.ds_fallbacks = 0;
  eps->stats.graph_segments = 0;
  eps->stats.gs_exact = 0;
  eps->stats.bytes_moved = 0.0;
  eps->stats.kernel_launches = 0;
  eps->stats.precision_steps = 0;
  eps->stats.precision_restarts = 0;
  eps->ev_cls.clear();
  eps->ev_used = 0;
  eps->solved = 0;
  int nconv = 0, its = 0, reason = 0;
  double bytes = 0.0;
  if (eps->arith != ARITH_F32) {
    KSG_TRY(eps_solve_core(eps, eps->tol_e, t0, &nconv, &its, &reason, &bytes));
  } else {
    // The precision form.  Phase 1 stores the operator values and the basis in FP32 (half the bytes) with every
    // product and sum accumulated exactly in pairs; its accuracy is limited by the FP32 basis (about 1e-7 relative),
    // so it runs to max(tol, 1e-6).  Each converged pair is then rechecked in FP64 (||A x - lambda x|| / |lambda|);
    // if one fails tol, an FP64-class refinement sweep -- a pair-storage Krylov-Schur solve started from the sum of
    // the phase-1 Ritz vectors, whose Krylov space already holds the wanted directions -- finishes to tol.
    const double tol1 = std::max(eps->tol_e, 1e-6);
    eps->storage = STORE_F32;
    KSG_TRY(eps_solve_core(eps, tol1, t0, &nconv, &its, &reason, &bytes));
    eps->stats.precision_steps = eps->stats.krylov_steps;
    eps->stats.precision_restarts = its;
    eps->nconv = nconv;
    eps->solved = 1;  // EPSComputeError reads the phase-1 results
    bool pass = reason == 1;
    const int check = std::min(nconv, eps->nev_e);
    for (int i = 0; i < check && pass; ++i) {
      double err = 0.0;
      KSG_TRY(EPSComputeError(eps, i, EPS_ERROR_RELATIVE, &err));
      if (!(err <= eps->tol_e)) pass = false;
    }
    eps->solved = 0;
    if (pass) {
      KSG_TRY(ksg_eps_widen_f32(eps, nconv));
      eps->storage = STORE_PAIR;
    } else {
      // start vector of the sweep: the sum of the phase-1 Ritz vectors of the wanted eigenvalues
      std::vector<double> acc(eps->n, 0.0), col(eps->n);
      const int use = std::max(1, std::min(nconv, eps->nev_e));
      for (int i = 0; i < use && i < nconv; ++i) {
        KSG_TRY(ksg_get_column(col.data(), ksg_col(eps->V.p, eps->ldv, eps->perm[i], STORE_F32), eps->n, STORE_F32,
                               s));
        for (int r = 0; r < eps->n; ++r) acc[r] += col[r];
      }
      eps->v0_internal.swap(acc);
      eps->storage = STORE_PAIR;
      int its2 = 0;
      double bytes2 = 0.0;
      PetscErrorCode ierr = eps_solve_core(eps, eps->tol_e, t0, &nconv, &its2, &reason, &bytes2);
      eps->v0_internal.clear();
      KSG_TRY(ierr);
      its += its2;
      bytes += bytes2;
    }
  }
  KSG_CUDA(cudaEventRecord(eps->ev_solve[1], s));
  KSG_CUDA(cudaStreamSynchronize(s));
  if (eps->rtc.count >= restart_t5_scratch_bytes(eps->ld)) {
    int flag = 0;  // a bounded wait of the tcgen05 restart ran out (the kernel freed its TMEM and returned)
    KSG_CUDA(cudaMemcpy(&flag, restart_t5_errflag(eps->rtc.p, eps->ld), sizeof(int), cudaMemcpyDeviceToHost));
    KSG_CHECK(!flag, PETSC_ERR_GPU, "tcgen05 restart: a bounded wait ran out; results are not valid");
  }
  if (eps->gs_tc_on) {
    int flag = 0;  // 1: a bounded wait of a tensor-core Gram-Schmidt kernel ran out; 2: a value reached its scale
    KSG_CUDA(cudaMemcpy(&flag, eps->gterr.p, sizeof(int), cudaMemcpyDeviceToHost));
    KSG_CHECK(flag != 1, PETSC_ERR_GPU, "tensor-core Gram-Schmidt: a bounded wait ran out; results are not valid");
    KSG_CHECK(flag != 2, PETSC_ERR_PLIB,
              "exact-product Gram-Schmidt: a basis value exceeded its recorded exponent; results are not valid");
  }
  {
    float ms = 0.0f;
    KSG_CUDA(cudaEventElapsedTime(&ms, eps->ev_solve[0], eps->ev_solve[1]));
    eps->stats.solve_device_ms = ms;
  }
  prof_collect(eps);
  eps->nconv = nconv;
  eps->its = its;
  eps->reason = reason;
  eps->solved = 1;
  eps->stats.bytes_moved = bytes;
  eps->stats.solve_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  if (!eps->post_views.empty()) KSG_TRY(ksg_eps_post_views(eps));
  return 0;
}

extern "C" PetscErrorCode EPSGetConverged(EPS eps, PetscInt *nconv) {
  KSG_CHECK(eps && nconv, PETSC_ERR_ARG_NULL, "Null argument");
  KSG_CHECK(eps->solved, PETSC_ERR_ORDER, "Must call EPSSolve() first");
  *nconv = eps->nconv;
  return 0;
}
extern "C" PetscErrorCode EPSGetConvergedReason(EPS eps, EPSConvergedReason *reason) {
  KSG_CHECK(eps && reason, PETSC_ERR_ARG_NULL, "Null argument");
  KSG_CHECK(eps->solved, PETSC_ERR_ORDER, "Must call EPSSolve() first");
  *reason = (EPSConvergedReason)eps->reason;
  return 0;
}
extern "C" PetscErrorCode EPSGetIterationNumber(EPS eps, PetscInt *its) {
  KSG_CHECK(eps && its, PETSC_ERR_ARG_NULL, "Null argument");
  *its = eps->its;
  return 0;
}
extern "C" PetscErrorCode EPSGetEigenvalue(EPS eps, PetscInt i, PetscScalar *eigr, PetscScalar *eigi) {
  KSG_CHECK(eps, PETSC_ERR_ARG_NULL, "Null EPS");
  KSG_CHECK(eps->solved, PETSC_ERR_ORDER, "Must call EPSSolve() first");
  KSG_CHECK(i >= 0, PETSC_ERR_ARG_OUTOFRANGE, "The index cannot be negative");
  KSG_CHECK(i < eps->nconv, PETSC_ERR_ARG_OUTOFRANGE, "The index can be nconv-1 at most, see EPSGetConverged()");
  const int k = eps->perm[i];
  if (eigr) *eigr = eps->r_eigr[k];
  if (eigi) *eigi = eps->r_eigi[k];
  return 0;
}
// BV_GetEigenvector (bvimpl.h:421-444)
extern "C" PetscErrorCode EPSGetEigenvector(EPS eps, PetscInt i, Vec Vr, Vec Vi) {
  KSG_CHECK(eps, PETSC_ERR_ARG_NULL, "Null EPS");
  KSG_CHECK(eps->solved, PETSC_ERR_ORDER, "Must call EPSSolve() first");
  KSG_CHECK(i >= 0 && i < eps->nconv, PETSC_ERR_ARG_OUTOFRANGE, "Index out of range");
  const int n = eps->n;
  KSG_CHECK((!Vr || Vr->n == n) && (!Vi || Vi->n == n), PETSC_ERR_ARG_SIZ, "Vector of the wrong size");
  const int k = eps->perm[i];
  const double ei = eps->r_eigi[k];
  const double *col = eps_basis(eps) + (size_t)k * eps->ldv;
  const size_t bytes = sizeof(double) * n;
  const int sto = eps->storage;
  if (ei > 0.0) {
    if (Vr) KSG_TRY(ksg_get_column(Vr->a, col, n, sto, eps->stream));
    if (Vi) KSG_TRY(ksg_get_column(Vi->a, col + eps->ldv, n, sto, eps->stream));
  } else if (ei < 0.0) {
    if (Vr) KSG_TRY(ksg_get_column(Vr->a, col - eps->ldv, n, sto, eps->stream));
    if (Vi) {
      KSG_TRY(ksg_get_column(Vi->a, col, n, sto, eps->stream));
      for (int r = 0; r < n; ++r) Vi->a[r] = -Vi->a[r];
    }
  } else {
    if (Vr) KSG_TRY(ksg_get_column(Vr->a, col, n, sto, eps->stream));
    if (Vi) memset(Vi->a, 0, bytes);
  }
  if (Vr && eps->B && eps->problem == EPS_GHEP) {
    if (eps->d_chol.p) {  // the basis holds y = L^T x: x = L^-T y on the device
      DBuf<double> t;
      KSG_CUDA(t.alloc(n));
      KSG_CUDA(cudaMemcpyAsync(t.p, Vr->a, bytes, cudaMemcpyHostToDevice, eps->stream));
      KSG_CUDA(launch_lt_solve(eps->d_chol.p, t.p, n, 1, n, eps->stream));
      KSG_CUDA(cudaMemcpyAsync(Vr->a, t.p, bytes, cudaMemcpyDeviceToHost, eps->stream));
      KSG_CUDA(cudaStreamSynchronize(eps->stream));
    } else {  // the basis holds y = D^1/2 x
      for (int r = 0; r < n; ++r) Vr->a[r] *= 1.0 / sqrt(eps->bdiag[r]);
    }
  }
  return 0;
}
extern "C" PetscErrorCode EPSGetEigenpair(EPS eps, PetscInt i, PetscScalar *eigr, PetscScalar *eigi, Vec Vr, Vec Vi) {
  KSG_TRY(EPSGetEigenvalue(eps, i, eigr, eigi));
  if (Vr || Vi) KSG_TRY(EPSGetEigenvector(eps, i, Vr, Vi));
  return 0;
}
extern "C" PetscErrorCode EPSGetErrorEstimate(EPS eps, PetscInt i, PetscReal *errest) {
  KSG_CHECK(eps && errest, PETSC_ERR_ARG_NULL, "Null argument");
  KSG_CHECK(eps->solved, PETSC_ERR_ORDER, "Must call EPSSolve() first");
  KSG_CHECK(i >= 0 && i < eps->nconv, PETSC_ERR_ARG_OUTOFRANGE, "Index out of range");
  *errest = eps->r_errest[eps->perm[i]];
  return 0;
}

// residual norms on the device: per block, the sums of (y - kr Bx + ki Bxi)^2, of (yi - kr Bxi - ki Bx)^2 and of
// x^2, FP64; b is the diagonal of B, or null for B = I
__global__ void k_residual(const double *y, const double *yi, const double *x, const double *xi, const double *b,
                           double kr, double ki, int n, double *part) {
  __shared__ double s0[256], s1[256], s2[256];
  double a0 = 0.0, a1 = 0.0, a2 = 0.0;
  for (long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (long long)gridDim.x * blockDim.x) {
    const double bx = b ? b[r] * x[r] : x[r];
    const double bxi = xi ? (b ? b[r] * xi[r] : xi[r]) : 0.0;
    double u = y[r] - kr * bx + (xi ? ki * bxi : 0.0);
    a0 = fma(u, u, a0);
    if (yi) {
      double v = yi[r] - kr * bxi - ki * bx;
      a1 = fma(v, v, a1);
    }
    a2 = fma(x[r], x[r], a2);
  }
  s0[threadIdx.x] = a0;
  s1[threadIdx.x] = a1;
  s2[threadIdx.x] = a2;
  __syncthreads();
  for (int off = 128; off > 0; off >>= 1) {
    if (threadIdx.x < off) {
      s0[threadIdx.x] += s0[threadIdx.x + off];
      s1[threadIdx.x] += s1[threadIdx.x + off];
      s2[threadIdx.x] += s2[threadIdx.x + off];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    part[3 * blockIdx.x] = s0[0];
    part[3 * blockIdx.x + 1] = s1[0];
    part[3 * blockIdx.x + 2] = s2[0];
  }
}

// x <- d .* x (the map y -> x = D^-1/2 y of EPS_GHEP)
__global__ void k_diag_mul(double *x, const double *d, int n) {
  for (long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (long long)gridDim.x * blockDim.x)
    x[r] *= d[r];
}

// EPSComputeError / EPSComputeResidualNorm_Private (epssolve.c:666-815): ||A x - k B x|| with the user's A and B;
// for EPS_GHEP the basis column holds y = D^1/2 x and the relative and backward errors divide by ||x||
extern "C" PetscErrorCode EPSComputeError(EPS eps, PetscInt i, EPSErrorType type, PetscReal *error) {
  KSG_CHECK(eps && error, PETSC_ERR_ARG_NULL, "Null argument");
  KSG_CHECK(eps->solved, PETSC_ERR_ORDER, "Must call EPSSolve() first");
  KSG_CHECK(i >= 0 && i < eps->nconv, PETSC_ERR_ARG_OUTOFRANGE, "Index out of range");
  const int n = eps->n;
  const int k = eps->perm[i];
  double kr = eps->r_eigr[k], ki = eps->r_eigi[k];
  const int kx = (ki < 0.0) ? k - 1 : k;  // the stored pair is (x, xi) for the eigenvalue with positive imaginary part
  const double *x = static_cast<const double *>(ksg_col(eps_basis(eps), eps->ldv, kx, eps->storage));
  const double *xi = (ki != 0.0) ? static_cast<const double *>(ksg_col(eps_basis(eps), eps->ldv, kx + 1, eps->storage))
                                  : nullptr;
  if (ki < 0.0) ki = -ki;
  const int gen = eps->B != nullptr;
  const int ghep = gen && eps->problem == EPS_GHEP;
  if (gen) KSG_TRY(ksg_mat_upload(eps->A));  // the iteration ran on the scaled operator
  DBuf<double> y, yi, part, xd, xid;
  const int blocks = std::min(1024, (n + 255) / 256);
  KSG_CUDA(y.alloc(n));
  if (xi) KSG_CUDA(yi.alloc(n));
  KSG_CUDA(part.alloc(3 * blocks));
  cudaStream_t s = eps->stream;
  if (eps->storage == STORE_F32) {
    KSG_CUDA(xd.alloc(n));
    KSG_CUDA(launch_f32_to_f64(reinterpret_cast<const float *>(x), xd.p, n, s));
    x = xd.p;
    if (xi) {
      KSG_CUDA(xid.alloc(n));
      KSG_CUDA(launch_f32_to_f64(reinterpret_cast<const float *>(xi), xid.p, n, s));
      xi = xid.p;
    }
  } else if (eps->storage == STORE_PAIR) {
    KSG_CUDA(xd.alloc(n));
    KSG_CUDA(launch_pair_to_f64(reinterpret_cast<const float2 *>(x), xd.p, n, s));
    x = xd.p;
    if (xi) {
      KSG_CUDA(xid.alloc(n));
      KSG_CUDA(launch_pair_to_f64(reinterpret_cast<const float2 *>(xi), xid.p, n, s));
      xi = xid.p;
    }
  } else if (ghep) {
    KSG_CUDA(xd.alloc(n));
    KSG_CUDA(cudaMemcpyAsync(xd.p, x, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
    x = xd.p;
  }
  if (ghep) {  // eigenvalues of EPS_GHEP are real: no xi
    if (eps->d_chol.p) {
      KSG_CUDA(launch_lt_solve(eps->d_chol.p, xd.p, n, 1, n, s));  // x = L^-T y
    } else {
      k_diag_mul<<<blocks, 256, 0, s>>>(xd.p, eps->d_bisqrt.p, n);
      KSG_CUDA(cudaGetLastError());
    }
  }
  const Mat A = eps->A;
  const int alanes = spmv_lanes_for((double)A->nnz / n);
  KSG_CUDA(launch_spmv(A->d_rp.p, A->d_ci.p, A->d_va.p, x, y.p, n, alanes, nullptr, 1.0, s));
  if (xi) KSG_CUDA(launch_spmv(A->d_rp.p, A->d_ci.p, A->d_va.p, xi, yi.p, n, alanes, nullptr, 1.0, s));
  DBuf<double> bx, bxi;
  double xnorm2 = -1.0;  // ||x||^2 when the residual kernel receives B x instead of x
  if (gen && eps->bdiag.empty()) {
    if (ghep) {
      k_residual<<<blocks, 256, 0, s>>>(x, nullptr, x, nullptr, nullptr, 0.0, 0.0, n, part.p);
      KSG_CUDA(cudaGetLastError());
      std::vector<double> hp(3 * blocks);
      KSG_CUDA(cudaMemcpyAsync(hp.data(), part.p, sizeof(double) * 3 * blocks, cudaMemcpyDeviceToHost, s));
      KSG_CUDA(cudaStreamSynchronize(s));
      xnorm2 = 0.0;
      for (int b = 0; b < blocks; ++b) xnorm2 += hp[3 * b];
    }
    // a non-diagonal B: the residual takes B x (and B xi) from its own product
    const Mat B = eps->B;
    KSG_TRY(ksg_mat_upload(B));
    const int blanes = spmv_lanes_for((double)B->nnz / n);
    KSG_CUDA(bx.alloc(n));
    KSG_CUDA(launch_spmv(B->d_rp.p, B->d_ci.p, B->d_va.p, x, bx.p, n, blanes, nullptr, 1.0, s));
    if (xi) {
      KSG_CUDA(bxi.alloc(n));
      KSG_CUDA(launch_spmv(B->d_rp.p, B->d_ci.p, B->d_va.p, xi, bxi.p, n, blanes, nullptr, 1.0, s));
    }
    x = bx.p;
    xi = xi ? bxi.p : nullptr;
  }
  k_residual<<<blocks, 256, 0, s>>>(y.p, xi ? yi.p : nullptr, x, xi,
                                    (gen && !eps->bdiag.empty()) ? eps->d_bdiag.p : nullptr, kr, ki, n, part.p);
  KSG_CUDA(cudaGetLastError());
  std::vector<double> h(3 * blocks);
  KSG_CUDA(cudaMemcpyAsync(h.data(), part.p, sizeof(double) * 3 * blocks, cudaMemcpyDeviceToHost, s));
  KSG_CUDA(cudaStreamSynchronize(s));
  double s0 = 0.0, s1 = 0.0, s2 = 0.0;
  for (int b = 0; b < blocks; ++b) {
    s0 += h[3 * b];
    s1 += h[3 * b + 1];
    s2 += h[3 * b + 2];
  }
  double nrm = xi ? hypot(sqrt(s0), sqrt(s1)) : sqrt(s0);
  const double lam = hypot(kr, ki);
  const double vecnorm = ghep ? sqrt(xnorm2 >= 0.0 ? xnorm2 : s2) : 1.0;  // epssolve.c:767
  switch (type) {
    case EPS_ERROR_ABSOLUTE: break;
    case EPS_ERROR_RELATIVE: nrm /= lam * vecnorm; break;
    case EPS_ERROR_BACKWARD:
      nrm /= (ksg_mat_norm_inf(A) + lam * (gen ? ksg_mat_norm_inf(eps->B) : 1.0)) * vecnorm;
      break;
    default: return ksg_set_error(PETSC_ERR_ARG_OUTOFRANGE, "Invalid error type");
  }
  *error = nrm;
  return 0;
}

extern "C" PetscErrorCode EPSGB300GetStats(EPS eps, EPSGB300Stats *stats) {
  KSG_CHECK(eps && stats, PETSC_ERR_ARG_NULL, "Null argument");
  *stats = eps->stats;
  return 0;
}

// Column i of X = the real eigenvector of pair i as EPSGetEigenvector(i) returns it; for a complex pair listed as
// i, i+1 the real part and the imaginary part (of the eigenvalue with positive imaginary part) in columns i and i+1,
// the layout of the reference's basis after EPSComputeVectors_Schur (epsdefault.c:105-169).  Values are converted
// to IEEE doubles from the basis' storage format and, for EPS_GHEP, mapped back from y = D^1/2 x.
__global__ void k_gather_eigvecs(const void *V, long long ldv, int storage, const int *cols, const double *bisqrt,
                                 int n, int nconv, double *X, long long ldx) {
  const int i = blockIdx.y;
  if (i >= nconv) return;
  const size_t k = (size_t)cols[i];
  for (long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (long long)gridDim.x * blockDim.x) {
    double v;
    if (storage == STORE_F64) v = static_cast<const double *>(V)[r + k * ldv];
    else if (storage == STORE_F32) v = (double)static_cast<const float *>(V)[r + k * ldv];
    else {
      const float2 p = static_cast<const float2 *>(V)[r + k * ldv];
      v = (double)p.x + (double)p.y;
    }
    if (bisqrt) v *= bisqrt[r];
    X[r + (size_t)i * ldx] = v;
  }
}

// the device-side counterpart of EPSGetEigenvector for every converged pair at once
extern "C" PetscErrorCode EPSGB300GetDeviceEigenvectors(EPS eps, const double **X, PetscInt *ld) {
  KSG_CHECK(eps && X && ld, PETSC_ERR_ARG_NULL, "Null argument");
  KSG_CHECK(eps->solved, PETSC_ERR_ORDER, "Must call EPSSolve() first");
  const int n = eps->n, m = eps->nconv;
  const long long ldx = ((long long)n + 63) / 64 * 64;
  if (!eps->xvec_valid) {
    KSG_CUDA(cudaSetDevice(eps->device));
    if (m > 0) {
      if (eps->xvec.count < (size_t)ldx * m) KSG_CUDA(eps->xvec.alloc((size_t)ldx * m));
      if (eps->d_perm.count < (size_t)m) KSG_CUDA(eps->d_perm.alloc(m));
      std::vector<int> cols(m);
      for (int i = 0; i < m; ++i) {
        const int k = eps->perm[i];
        cols[i] = k;
        // the second of a complex pair follows its first: column k holds the imaginary part; a conjugate listed
        // without its partner just before it gives its real part, column k - 1
        if (eps->r_eigi[k] < 0.0 && !(i > 0 && eps->perm[i - 1] == k - 1)) cols[i] = k - 1;
      }
      KSG_CUDA(cudaMemcpyAsync(eps->d_perm.p, cols.data(), sizeof(int) * m, cudaMemcpyHostToDevice, eps->stream));
      const double *bis = (eps->B && eps->problem == EPS_GHEP) ? eps->d_bisqrt.p : nullptr;
      dim3 grid((unsigned)std::min<long long>((n + 255) / 256, 1024), (unsigned)m);
      k_gather_eigvecs<<<grid, 256, 0, eps->stream>>>(eps_basis(eps), eps->ldv, eps->storage, eps->d_perm.p, bis, n, m,
                                                      eps->xvec.p, ldx);
      KSG_CUDA(cudaGetLastError());
      if (eps->B && eps->problem == EPS_GHEP && eps->d_chol.p)  // x = L^-T y for every column
        KSG_CUDA(launch_lt_solve(eps->d_chol.p, eps->xvec.p, n, m, ldx, eps->stream));
      KSG_CUDA(cudaStreamSynchronize(eps->stream));
    }
    eps->xvec_valid = 1;
  }
  *X = eps->xvec.p;
  *ld = (PetscInt)ldx;
  return 0;
}

// kept for existing callers: the same FP64 eigenvector array as EPSGB300GetDeviceEigenvectors
extern "C" PetscErrorCode EPSGB300GetDeviceBasis(EPS eps, const double **V, PetscInt *ld) {
  return EPSGB300GetDeviceEigenvectors(eps, V, ld);
}

// ||V^T V - I||_max over the first nconv columns (solver order), with the GS_DOTS kernel in the EPS arithmetic
extern "C" PetscErrorCode EPSGB300OrthogonalityError(EPS eps, PetscReal *err) {
  KSG_CHECK(eps && err, PETSC_ERR_ARG_NULL, "Null argument");
  KSG_CHECK(eps->solved, PETSC_ERR_ORDER, "Must call EPSSolve() first");
  const int m = eps->nconv;
  double worst = 0.0;
  StepArgs a = {};
  a.V = eps_basis(eps);
  a.ldv = eps->ldv;
  a.n = eps->n;
  a.coef = eps->coef.p;
  a.part = eps->part.p;
  a.pstride = eps->pstride;
  a.st = eps->st.p;
  a.eta = 0.7071;
  std::vector<double> h(eps->ld + 1);
  for (int j = 0; j < m; ++j) {
    KSG_CUDA(launch_segment_begin(eps->st.p, 0, 0, eps->stream));
    a.J = j;
    a.j = j;
    a.U = eps_basis(eps) + (size_t)j * eps->ldv;
    KSG_CUDA(launch_gs_dot(a, 1, GS_DOTS, eps->storage == STORE_PAIR ? ARITH_PAIR : ARITH_F64, eps->stream,
                           eps->storage));
    KSG_CUDA(cudaMemcpyAsync(h.data(), eps->coef.p, sizeof(double) * (j + 1), cudaMemcpyDeviceToHost, eps->stream));
    KSG_CUDA(cudaStreamSynchronize(eps->stream));
    for (int i = 0; i < j; ++i) worst = std::max(worst, fabs(h[i]));
    worst = std::max(worst, fabs(h[j] - 1.0));
  }
  *err = worst;
  return 0;
}
