// kernels.h -- host-side launchers of the CUDA kernels (no CUDA types beyond cudaStream_t / cudaError_t).
#pragma once

#include <cuda_runtime.h>

#include <cfloat>

#include "ks_types.h"

namespace ksg {

// Arguments of the projected-problem kernels.
struct DSArgs {
  int ld;          // leading dimension of Q / H (ncv + 1)
  int n;           // problem size when st is NULL (DS API); otherwise st->m is used
  int flags;       // DS_DO_* operations to run
  int l;           // locked columns (nconv)
  int k;           // nconv + kept columns (start of the new Krylov segment)
  int raw;         // 1 if the matrix still holds the arrow / Krylov-Schur form (kept columns > 0)
  double *d, *e;   // symmetric: diagonal and off-diagonal / extra row (length ld)
  double *H;       // non-symmetric: ld x ld matrix, extra row at row n
  double *Q;       // ld x ld
  double *eigr, *eigi, *errest;  // length ld
  double *work;    // scratch (non-symmetric solver), 4 * ld doubles
  int which;
  double tol;
  int nev, its, max_it;
  double keep;
  int lock;
  const KrylovState *st;
  KSControl *ctl;
  double target;   // target of the EPS_TARGET_* criteria (operator scale applied)
  int harmonic;    // non-symmetric solver: harmonic Rayleigh-Ritz translation for the target
  int conv;        // DS_CONV_*: the error estimate of the convergence test
  double conv_a, conv_b;  // DS_CONV_ABS: res / conv_a; DS_CONV_NORM: res / (conv_a + conv_b |k|)
  const int *run_if = nullptr;  // the FP64 QR kernel runs only when this device flag is nonzero (null: always)
};

// convergence tests (EPSConvergedRelative / Absolute / Norm, epsdefault.c:224-256) on the scaled operator: the
// residual norm res and the eigenvalue modulus w are both scaled by the operator scale s, so ABS divides by s and
// NORM by ||A|| s + ||B|| w
enum { DS_CONV_REL = 0, DS_CONV_ABS = 1, DS_CONV_NORM = 2 };
#ifdef __CUDACC__
__device__ __forceinline__ double ds_conv_errest(const DSArgs &a, double res, double w) {
  if (a.conv == DS_CONV_REL) return (w != 0.0) ? res / w : DBL_MAX;
  const double den = (a.conv == DS_CONV_ABS) ? a.conv_a : a.conv_a + a.conv_b * w;
  return (den != 0.0) ? res / den : DBL_MAX;
}
#endif

enum { DS_DO_SOLVE = 1, DS_DO_SORT = 2, DS_DO_EXTRAROW = 4, DS_DO_CONTROL = 8, DS_DO_ALL = 15 };

// Scratch of the mixed-precision symmetric projected solver (k_ds_fast.cu): five ld x ld FP64 matrices and a few
// vectors, carved from one allocation by ds_fast_layout.  The problem fields are filled from DSArgs at launch.
struct DSFArgs {
  int ld, n, l, k, raw;
  const double *d, *e;
  double *T, *X, *P, *S, *G;  // ld x ld: projected matrix, eigenvectors, product, X^T T X, X^T X
  double *W;                  // 2 * ld * 16: cluster rotations and cluster blocks
  double *lam, *part, *scal;  // eigenvalue estimates, block partial sums, thresholds
  int *fallback;              // set by the final step when the refined pairs fail the accuracy check
  const KrylovState *st;
  KSControl *ctl;
};

// Rows of the operator longer than long_t nonzeros, cut into segments of at most LONG_SEG nonzeros: each segment is
// summed by one warp, then each long row merges its segments in order (deterministic, no atomics).  Built once per
// matrix (ksg_mat_upload); `part` is per-solver scratch (one 8-byte partial per segment).
constexpr int LONG_ROW_T = 4096;
constexpr int LONG_SEG = 2048;
struct LongRows {
  int n_long = 0, n_seg = 0, long_t = 0x7fffffff;
  const int *seg_row = nullptr, *seg_beg = nullptr, *seg_end = nullptr;  // per segment
  const int *lrow = nullptr, *lfirst = nullptr;                           // per long row: row, first segment
  void *part = nullptr;
};

// The Gram-Schmidt pair for IEEE-double storage on the tensor cores (k_gs_tc.cu).  The basis columns' scales live in
// an int8 table [column][128-row tile] (leading dimension ldt, a multiple of 8): the update half and the tcgen05
// restart record the exponents of the columns they write.
struct GTArgs {
  signed char *vexp;  // exponent e of each (column, tile): every |v| < 2^e there; -128 for an all-zero tile
  int ldt;            // tiles per column in the table (a multiple of 8)
  int ct;             // half A: tiles per chunk (set by the launcher)
  double *part;       // per-block partials (gs_tc_part_doubles() doubles)
  int pstride;        // half A: doubles per block in part (set by the launcher)
  int *err;           // set to 1 when a bounded wait ran out, to 2 when a value reached its recorded scale
  int integer;        // 1: the integer-pipe kernels (k_gs_ix.cu) instead of the tensor-core ones
};
int gs_tc_max_columns();
size_t gs_tc_part_doubles();
cudaError_t launch_gs_dot_tc(const StepArgs &a, int nx, int mode, const GTArgs &g, cudaStream_t s);
cudaError_t launch_gs_update_tc(const StepArgs &a, int nx, int mode, const GTArgs &g, cudaStream_t s);
// the same pair with exact products on the integer pipes (k_gs_ix.cu): the same exponent table, partials and flag
int gs_ix_max_columns();
cudaError_t launch_gs_dot_ix(const StepArgs &a, int nx, int mode, const GTArgs &g, cudaStream_t s);
cudaError_t launch_gs_update_ix(const StepArgs &a, int nx, int mode, const GTArgs &g, cudaStream_t s);
// the exponents of the 128-row tiles of one IEEE-double column (vexp_col = the table row of that column)
cudaError_t launch_record_vexp(const double *col, int n, signed char *vexp_col, cudaStream_t s);

int num_sms();
int spmv_lanes_for(double avg_nnz);
int gs_dot_blocks(int n);
int gs_update_blocks(int n);
int gs_max_columns();  // columns of the register-tiled dot kernel; wider bases take the column-group kernel
int gs_wide_max_columns();
size_t restart_smem_bytes(int K, int N, int tile_rows);
int restart_wide_max_columns();

cudaError_t launch_spmv(const int *rp, const int *ci, const double *va, const double *x, double *y, int n, int lanes,
                        const KrylovState *st, double scale, cudaStream_t s);
cudaError_t launch_spmv_storage(const int *rp, const int *ci, const double *va, const float2 *va_pair, const void *x,
                                void *y, int n, int lanes, const KrylovState *st, double scale, int storage,
                                cudaStream_t s, const LongRows *lr = nullptr, const float *va32 = nullptr);
cudaError_t launch_f64_to_pair(const double *x, float2 *y, long long n, cudaStream_t s);
cudaError_t launch_pair_to_f64(const float2 *x, double *y, long long n, cudaStream_t s);
cudaError_t launch_f64_to_f32(const double *x, float *y, long long n, cudaStream_t s);
cudaError_t launch_f32_to_f64(const float *x, double *y, long long n, cudaStream_t s);
// max_blocks > 0 caps the grid (the blocks loop over the row tiles, so any grid size gives the same sums' partition
// per block count)
cudaError_t launch_gs_dot(const StepArgs &a, int nx, int mode, int arith, cudaStream_t s, int storage = STORE_F64,
                          int max_blocks = 0);
cudaError_t launch_gs_update(const StepArgs &a, int nx, int mode, int arith, cudaStream_t s, int storage = STORE_F64);
cudaError_t launch_restart(void *V, long long ldv, int n, int a0, int K, int s0, int N, const double *Q, int ldq,
                           int arith, cudaStream_t s, int storage = STORE_F64);
// the restart on the bf16 tensor cores (pair storage, k_restart_tc.cu); scratch of restart_tc_scratch_bytes(ld)
size_t restart_tc_scratch_bytes(int ld);
// the same restart on tcgen05 (TMEM accumulators), bit-identical results; scratch of restart_t5_scratch_bytes(ld),
// zeroed once (it holds the flag restart_t5_errflag, set when a bounded wait of the kernel ran out)
size_t restart_t5_scratch_bytes(int ld);
int *restart_t5_errflag(void *scratch, int ld);
cudaError_t launch_restart_t5(float2 *V, long long ldv, int n, int a0, int K, int s0, int N, const double *Q, int ldq,
                              void *scratch, int ld, cudaStream_t s);
// the tcgen05 restart for FP64 storage: Q in 8 slices (7 when K > 128), the exact level sums rounded once to
// doubles; the same scratch and timeout flag
cudaError_t launch_restart_t5_f64(double *V, long long ldv, int n, int a0, int K, int s0, int N, const double *Q,
                                  int ldq, void *scratch, int ld, cudaStream_t s, signed char *vexp = nullptr,
                                  int ldt = 0);
cudaError_t launch_restart_tc(float2 *V, long long ldv, int n, int a0, int K, int s0, int N, const double *Q, int ldq,
                              void *scratch, int ld, cudaStream_t s);
cudaError_t launch_segment_begin(KrylovState *st, int k0, int m, cudaStream_t s);
cudaError_t launch_set_unit_scale(KrylovState *st, cudaStream_t s);
cudaError_t launch_set_scales(KrylovState *st, double sigma, double invnu, cudaStream_t s);
cudaError_t launch_scale(double *x, int n, double alpha, cudaStream_t s);
cudaError_t launch_negate(void *x, long long count, int as_float, cudaStream_t s);
// n_max <= 144: Q in shared memory; up to ds_hep_max_n(): Q rotated in place in a.Q (a.ld >= n_max)
cudaError_t launch_ds_hep(const DSArgs &a, int n_max, cudaStream_t s);
int ds_hep_max_n();
// n_max <= 144: A (and Q when it fits) in shared memory; up to ds_nhep_max_n(): in place in a.H and a.Q
cudaError_t launch_ds_nhep(const DSArgs &a, int n_max, cudaStream_t s);
int ds_nhep_max_n();
cudaError_t prepare_ds_nhep();  // shared-memory attributes of the NHEP solver kernels (call outside graph capture)
size_t ds_fast_scratch_doubles(int ld);
DSFArgs ds_fast_layout(double *scratch, int ld);
int ds_fast_launches();
// full DS_DO_ALL contract of launch_ds_hep for the Krylov-Schur loop (a.st and a.ctl required)
cudaError_t launch_ds_hep_fast(const DSArgs &a, const DSFArgs &f, int n_max, cudaStream_t s);
cudaError_t launch_nhep_vectors(double *T, int ld, int n, double *X, cudaStream_t s);
// C = B^-1 A for a non-diagonal B (k_dense.cu): Bd and Cd are n x n device scratch (row-major; Cd returns C), piv n
// ints, *err zeroed by the caller (set to k + 1 at a zero pivot); n <= general_b_max_n()
cudaError_t launch_general_b_operator(const int *arp, const int *aci, const double *ava, const int *brp,
                                      const int *bci, const double *bva, int n, double *Bd, double *Cd, int *piv,
                                      int *err, cudaStream_t s);
int general_b_max_n();
// EPS_GHEP with a non-diagonal B = L L^T: Ld returns L (row-major, lower), Td returns C = L^-1 A L^-T (row-major,
// symmetric); Cd is scratch; *err = k + 1 when B is not positive definite
cudaError_t launch_general_b_ghep(const int *arp, const int *aci, const double *ava, const int *brp, const int *bci,
                                  const double *bva, int n, double *Ld, double *Cd, double *Td, int *err,
                                  cudaStream_t s);
cudaError_t launch_lt_mv(const double *L, const double *x, double *y, int n, cudaStream_t s);  // y = L^T x
// X <- L^-T X for m column-major vectors of leading dimension ldx (x = L^-T y: the eigenvectors of the pencil)
cudaError_t launch_lt_solve(const double *L, double *X, int n, int m, long long ldx, cudaStream_t s);

}  // namespace ksg
