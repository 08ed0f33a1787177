// internal.h -- object layouts and helpers shared by the C-API translation units.
#pragma once

#include <cuda_runtime.h>

#include <array>
#include <cstdio>
#include <map>
#include <string>
#include <vector>

#include "kernels.h"
#include "ks_types.h"
#include "../../include/slepc_gb300.h"

// ---------------------------------------------------------------------------------------------------------------
// error handling: every entry point returns a PETSc error code and records a message for PetscGB300LastError()
// ---------------------------------------------------------------------------------------------------------------
PetscErrorCode ksg_set_error(PetscErrorCode code, const char *fmt, ...);

#define KSG_CHECK(cond, code, ...)                                     \
  do {                                                                 \
    if (!(cond)) return ksg_set_error((code), __VA_ARGS__);            \
  } while (0)

#define KSG_CUDA(call)                                                                                     \
  do {                                                                                                     \
    cudaError_t e_ = (call);                                                                               \
    if (e_ != cudaSuccess)                                                                                 \
      return ksg_set_error(e_ == cudaErrorMemoryAllocation ? PETSC_ERR_GPU_RESOURCE : PETSC_ERR_GPU,       \
                           "CUDA error %s at %s:%d: %s", cudaGetErrorName(e_), __FILE__, __LINE__,         \
                           cudaGetErrorString(e_));                                                         \
  } while (0)

#define KSG_TRY(call)                          \
  do {                                         \
    PetscErrorCode ierr_ = (call);             \
    if (ierr_) return ierr_;                   \
  } while (0)

// device buffer with RAII release
template <class T>
struct DBuf {
  T *p = nullptr;
  size_t count = 0;
  cudaError_t alloc(size_t n) {
    release();
    if (n == 0) return cudaSuccess;
    cudaError_t e = cudaMalloc((void **)&p, n * sizeof(T));
    if (e == cudaSuccess) count = n;
    else p = nullptr;
    return e;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    count = 0;
  }
  ~DBuf() { release(); }
};

// one MatSetValue(s) entry waiting for MatAssemblyEnd
struct MatEntry {
  int row, col;
  double v;
  int add;  // ADD_VALUES (else INSERT_VALUES)
};

// the first word of every EPS, ST and Mat (PetscObjectSetName, PetscObjectTypeCompare read it)
constexpr unsigned KSG_EPS_COOKIE = 0x31535045u, KSG_ST_COOKIE = 0x31315453u, KSG_MAT_COOKIE = 0x3154414Du;

struct _p_Mat {
  unsigned cookie = KSG_MAT_COOKIE;
  int m = 0, n = 0;
  int dense = 0;
  int empty = 0;  // created by MatCreate, not yet filled (MatLoad, or MatSetSizes + MatSetValues + assembly)
  int sized = 0;  // MatSetSizes given
  std::vector<MatEntry> pending;  // MatSetValue(s) since the last assembly
  // AIJ (caller-owned arrays, or the own_* arrays of a loaded matrix)
  const PetscInt *ai = nullptr, *aj = nullptr;
  const PetscScalar *aa = nullptr;
  long long nnz = 0;
  std::vector<PetscInt> own_i, own_j;
  std::vector<double> own_a;
  // dense
  std::vector<double> dbuf;
  double *data = nullptr;
  int lda = 0;
  int refs = 1;
  // device copy of the CSR arrays (uploaded on first use by a solver)
  DBuf<int> d_rp, d_ci;
  DBuf<double> d_va;
  DBuf<float2> d_va2;  // values as FP32 pairs, for the pair-storage SpMV
  DBuf<float> d_va32;  // values rounded to FP32, for the precision form
  // rows longer than LONG_ROW_T nonzeros, cut into segments (the skew-aware SpMV of kernels.h)
  DBuf<int> d_seg_row, d_seg_beg, d_seg_end, d_lrow, d_lfirst;
  int n_long = 0, n_seg = 0;
  int device_ready = 0;
  double norm_inf = -1.0;
  long long state = 0;  // bumped when the values change (assembly, MatLoad, MatScale, ...)
};

struct _p_PetscViewer {
  FILE *f = nullptr;
  PetscFileMode mode = FILE_MODE_READ;
  std::string name;
  int ascii = 0;     // PETSCVIEWERASCII (text reports) rather than PETSCVIEWERBINARY
  int borrowed = 0;  // the process-wide stdout viewer: never closed, PetscViewerDestroy only clears the handle
  std::vector<PetscViewerFormat> formats;  // PetscViewerPushFormat stack
};

struct _p_Vec {
  int n = 0;
  std::vector<double> own;
  double *a = nullptr;
  double *placed_from = nullptr;  // VecPlaceArray: the array to return to at VecResetArray
};


// device helpers used by more than one object
PetscErrorCode ksg_mat_upload(Mat A);
double ksg_mat_norm_inf(Mat A);
PetscErrorCode ksg_random_fill(double *host, int n, unsigned long long seed, unsigned long long stream_index);

struct _p_DS;
struct _p_BV;
struct _p_ST {
  unsigned cookie = KSG_ST_COOKIE;
  EPS eps = nullptr;  // the owner
  int typeset = 0;    // STSetType, EPSSetFromOptions or EPSSetUp gave the type (STSHIFT)
};



// a report EPSSolve prints when it ends (options -eps_converged_reason, -eps_error_*, -eps_view_values)
struct EPSPostView {
  int kind;  // 0 converged reason, 1 error view (etype), 2 values view, 3 EPSView
  int etype;
  PetscViewerFormat format;
  std::string file;  // empty: stdout
};

struct _p_EPS {
  unsigned cookie = KSG_EPS_COOKIE;
  std::string name;    // PetscObjectSetName
  std::string prefix;  // EPSSetOptionsPrefix
  // configuration
  Mat A = nullptr;
  Mat B = nullptr;  // generalised problems: a diagonal B (EPSSetOperators)
  int problem = 0;  // EPSProblemType
  std::string type = "krylovschur";
  int which = 0;
  int nev = 1, ncv = PETSC_DETERMINE, mpd = PETSC_DETERMINE;
  double tol = PETSC_DETERMINE;
  int max_it = PETSC_DETERMINE;
  double keep = 0.5;
  int lock = 1;
  int extraction = 0;  // EPSExtraction: EPS_RITZ or EPS_HARMONIC
  double target = 0.0;
  int conv = EPS_CONV_REL;  // EPSConv
  int purify = 1;           // EPSSetPurify: GHEP eigenvectors x <- B^-1 A x, B-normalised
  int balance = 0, balance_its = 5;  // EPSSetBalance: EPS_BALANCE_NONE, 5 iterations, cutoff 1e-8 (epsbasic.c:72-74)
  double balance_cutoff = 1e-8;
  int trackall = 0;         // EPSSetTrackAll (stored; every current estimate is computed anyway)
  int arith = ksg::ARITH_PAIR;
  int storage = ksg::STORE_PAIR;  // basis format: pairs with pair arithmetic, doubles with FP64 arithmetic
  int ds_method = EPS_GB300_DS_AUTO;  // EPSGB300DSMethod
  int gs_method = EPS_GB300_GS_AUTO;  // EPSGB300GSMethod
  double time_limit = 0.0;        // EPSGB300SetTimeLimit (0: none)
  int restart_method = 0;         // EPSGB300RestartMethod
  int device = -1;
  std::vector<double> v0;  // the first vector of the initial space
  int nini = 0;            // the size of the initial space given
  std::vector<double> v0_internal;  // start vector of the precision form's refinement sweep
  unsigned long long seed = 0x5EEDULL;
  unsigned long long rng_counter = 0;
  // state
  int setup = 0, solved = 0;
  int n = 0, ncv_e = 0, mpd_e = 0, maxit_e = 0, nev_e = 0, ld = 0;
  double tol_e = 1e-8;
  double opscale = 1.0;
  // the operator the Krylov iteration runs on: A itself, or for a generalised problem with diagonal B a scaled
  // copy owned by the EPS (GHEP: D^-1/2 A D^-1/2 with D = B; GNHEP: D^-1 A)
  Mat op = nullptr;
  std::vector<double> bdiag;       // the diagonal of B (generalised problems)
  DBuf<double> d_bdiag, d_bisqrt;  // device copies of diag(B) and diag(B)^-1/2
  DBuf<double> d_chol;             // EPS_GHEP with a non-diagonal B = L L^T: L (row-major, lower); the basis holds L^T x
  double nrma = 0.0, nrmb = 0.0;   // infinity norms for EPS_CONV_NORM (nrmb stays 0 for standard problems)
  long long a_state = -1, b_state = -1;  // the matrices' states at EPSSetUp
  int lanes = 8;
  long long ldv = 0;
  cudaStream_t stream = nullptr;
  DBuf<double> V, d, e, H, Q, X, eigr, eigi, errest, coef, work, dsf;
  DBuf<double> seg_part;  // one 8-byte partial per long-row segment of the operator
  DBuf<signed char> vexp;  // tensor-core Gram-Schmidt: exponents of the basis columns per 128-row tile
  DBuf<double> gtpart;     // its per-block partials
  DBuf<int> gterr;         // its error flag
  ksg::GTArgs gt = {};
  int gs_tc_on = 0;        // the current solve runs the tensor-core Gram-Schmidt
  // EPSSetDeflationSpace: the vectors as given (ndefl x n, host) and, after EPSSetUp, the orthonormal constraint
  // columns kept from them (columns 0..nc-1 of V, ahead of the Krylov basis)
  std::vector<double> defl;
  int ndefl = 0, nc = 0;
  DBuf<double> xvec;      // EPSGB300GetDeviceEigenvectors: FP64 eigenvectors in EPSGetEigenpair order
  DBuf<int> d_perm;       // its column map
  int xvec_valid = 0;     // xvec holds the current solve's vectors
  // factorisation segments captured as CUDA graphs, keyed by (k, nv, storage, arithmetic)
  struct SegGraph {
    cudaGraphExec_t exec = nullptr;
    int seen = 0;               // direct runs so far (captured on the second)
    long long launches = 0;     // kernels in the graph
    double bytes = 0.0;         // algorithmic bytes of the segment
  };
  std::map<std::array<int, 4>, SegGraph> seg_graphs;
  int graph_mode = -1;  // EPSGB300SetGraphCapture
  DBuf<unsigned char> rtc;  // slices of Q for the tensor-core restart
  DBuf<float2> part;
  int pstride = 0;
  DBuf<ksg::KrylovState> st;
  DBuf<ksg::KSControl> ctl;
  ksg::KSControl *h_ctl = nullptr;  // pinned
  cudaEvent_t ev_solve[2] = {nullptr, nullptr};

  // results
  int nconv = 0, its = 0, reason = 0;
  std::vector<double> r_eigr, r_eigi, r_errest;
  std::vector<int> perm;
  EPSGB300Stats stats = {};
  // profiling: event pairs per launch, per kernel class
  int prof = 0;
  std::vector<cudaEvent_t> ev_pool;
  size_t ev_used = 0;
  std::vector<std::pair<int, double>> ev_cls;  // class and bytes of each recorded pair
  double prof_ms[EPS_GB300_K_COUNT] = {0};
  double prof_bytes[EPS_GB300_K_COUNT] = {0};
  long long prof_launches[EPS_GB300_K_COUNT] = {0};
  BV bv = nullptr;
  DS ds = nullptr;
  _p_ST stobj;  // EPSGetST
  // monitors (EPSMonitorSet) and the reports to print at the end of EPSSolve
  std::vector<EPSMonitorFn *> mon;
  std::vector<void *> mon_ctx;
  std::vector<PetscCtxDestroyFn *> mon_destroy;
  std::vector<EPSPostView> post_views;
};

// the Lanczos (symmetric) variant runs for EPS_HEP with Ritz extraction; harmonic extraction runs the Arnoldi
// variant with the non-symmetric projected solver (krylovschur.c:238-239)
// the largest leading dimension of the host-side DS object (DSAllocate); the solver's projected problems live on
// the device and have no such limit
constexpr int KSG_HOST_DS_MAX_LD = 144;

inline int ksg_eps_hermitian(EPS e) { return e->problem == EPS_HEP || e->problem == EPS_GHEP; }
inline int ksg_eps_lanczos(EPS e) { return ksg_eps_hermitian(e) && e->extraction != EPS_HARMONIC; }

// run the Gram-Schmidt pair kernels on one column (orthonormalise u = V[:, j] against V[:, 0:j]); returns the
// norm of the orthogonalised vector in *nrm and the linear-dependence flag (two CGS passes)
PetscErrorCode ksg_orthonormalize_column(void *V, long long ldv, int n, int j, double *coef, float2 *part,
                                         int pstride, ksg::KrylovState *st, int arith, cudaStream_t s, double *nrm,
                                         int *lindep, int refine, int storage = ksg::STORE_F64,
                                         const ksg::GTArgs *tc = nullptr);
PetscErrorCode ksg_mat_upload_pairs(Mat A);
PetscErrorCode ksg_mat_upload_f32(Mat A);
// address of basis column j for the storage format (8 bytes per entry, 4 for STORE_F32; same leading dimension)
inline size_t ksg_entry_bytes(int storage) { return storage == ksg::STORE_F32 ? 4 : 8; }
void *ksg_col(void *V, long long ldv, int j, int storage);
// host -> device copy of a double vector into a basis column of the given storage format
PetscErrorCode ksg_put_column(void *dst, const double *src, int n, int storage, cudaStream_t s);
// device basis column -> host doubles
PetscErrorCode ksg_get_column(double *dst, const void *src, int n, int storage, cudaStream_t s);
// pieces of EPSSolve shared with the batched engine (api_batch.cu)
PetscErrorCode ksg_eps_put_start(EPS eps, cudaStream_t s);
PetscErrorCode ksg_eps_widen_f32(EPS eps, int m);  // basis columns [0, m): FP32 -> pairs, in place
PetscErrorCode ksg_eps_new_start_vector(EPS eps, int col, int *breakdown);
PetscErrorCode ksg_eps_assemble(EPS eps, int nconv, const double *er, const double *ei, const double *es,
                                cudaStream_t s);
size_t ksg_part_stride(int ld);
// options support (api_io.cu): a viewer from "[ascii][:file][:format]"; a built-in monitor (kind 0 first, 1 all,
// 2 converged); the reports requested for the end of EPSSolve
PetscErrorCode ksg_viewer_from_spec(const char *spec, PetscViewer *viewer, PetscViewerFormat *format, int *ok);
PetscErrorCode ksg_eps_monitor_from_spec(EPS eps, int kind, const char *spec);
PetscErrorCode ksg_eps_post_views(EPS eps);
size_t ksg_part_blocks(int n);
