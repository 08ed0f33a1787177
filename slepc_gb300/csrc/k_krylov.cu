// k_krylov.cu -- the Krylov factorisation kernels of the GB300 Krylov-Schur path.
//
//   k_spmv          y = sigma * A x                CSR, sub-warp per row, FP64 FMA    (MatMult, bvops.c:862-885)
//   k_gs_dot        h = V^T [u w], u.u, u.w, w.w    half A of the Gram-Schmidt pair   (BVDotVec, bvblas.c:240-261)
//   k_gs_update     [v w'] = [u w] - V [s g]        half B of the Gram-Schmidt pair   (BVMultVec, bvblas.c:56-67)
//   k_restart       V(:,s:e) = V(:,a:b) Q(a:b,s:e)  thick restart, in place by rows    (BVMultInPlace, bvblas.c:74-106)
//
// Orthogonalisation is classical Gram-Schmidt with reorthogonalisation, arranged as DCGS2 (Bielich, Langou,
// Thomas, Swirydowicz, Yamazaki, Boman, "Low-synch Gram-Schmidt with delayed reorthogonalization for Krylov
// solvers", Parallel Computing 112, 2022): the reorthogonalisation of u_j is fused with the projection of
// w = A u_j, so each Krylov step reads the basis twice (once per kernel) instead of four times.  The Hessenberg
// column of A v_j is recovered as ([V_j^T w; v_j^T w] - H s) / nu, with u_j = nu v_j + V_j s.  Reductions are
// deterministic: fixed row partition, fixed-order merge of per-block partials by the last block to finish.
#include "common.cuh"
#include "kernels.h"
#include "krylov_body.cuh"
#include "ks_types.h"

#include <algorithm>

namespace ksg {

__global__ void k_f64_to_pair(const double *x, float2 *y, long long n) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const double v = x[i];
    const float hi = __double2float_rn(v);
    y[i] = make_float2(hi, __double2float_rn(v - (double)hi));
  }
}

__global__ void k_pair_to_f64(const float2 *x, double *y, long long n) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    y[i] = (double)x[i].x + (double)x[i].y;
}

// ------------------------------------------------------------------------------------------------------------
// Small helpers
// ------------------------------------------------------------------------------------------------------------
__global__ void k_segment_begin(KrylovState *st, int k0, int m) {
  st->sigma = 1.0;
  st->beta_prev = 0.0;
  st->invnu = 1.0;
  st->tau_sigma = 0.0;
  st->beta_out = 0.0;
  st->onorm = 0.0;
  st->stop = 0;
  st->m = m;
  st->breakdown = 0;
  st->k0 = k0;
}

__global__ void k_set_scales(KrylovState *st, double sigma, double invnu) {
  st->sigma = sigma;
  st->invnu = invnu;
  st->stop = 0;
}

__global__ void k_negate(double *x, long long n) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    x[i] = -x[i];
}
__global__ void k_negate_f32(float *x, long long n) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    x[i] = -x[i];
}

__global__ void k_scale_col(double *x, int n, double alpha) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    x[i] *= alpha;
}

// ------------------------------------------------------------------------------------------------------------
// Host-side launchers
// ------------------------------------------------------------------------------------------------------------
static int g_num_sms = 0;

int num_sms() {
  if (!g_num_sms) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, dev);
    if (g_num_sms <= 0) g_num_sms = 1;
  }
  return g_num_sms;
}

// threads per row: one thread per row for short rows (one FP64/pair FMA per nonzero, no shuffles), wider groups
// for long rows
int spmv_lanes_for(double avg_nnz) {
  if (avg_nnz <= 16.0) return 1;
  if (avg_nnz <= 64.0) return 8;
  return 32;
}

template <class S>
static void spmv_dispatch(const int *rp, const int *ci, const double *va, const void *x, void *y, int n, int lanes,
                          const KrylovState *st, double scale, int blocks, cudaStream_t s, int long_t) {
  using T = typename S::T;
  const T *xx = static_cast<const T *>(x);
  T *yy = static_cast<T *>(y);
  switch (lanes) {
    case 1: k_spmv<1, S><<<blocks, 256, 0, s>>>(rp, ci, va, xx, yy, n, st, scale, long_t); break;
    case 2: k_spmv<2, S><<<blocks, 256, 0, s>>>(rp, ci, va, xx, yy, n, st, scale, long_t); break;
    case 4: k_spmv<4, S><<<blocks, 256, 0, s>>>(rp, ci, va, xx, yy, n, st, scale, long_t); break;
    case 8: k_spmv<8, S><<<blocks, 256, 0, s>>>(rp, ci, va, xx, yy, n, st, scale, long_t); break;
    case 16: k_spmv<16, S><<<blocks, 256, 0, s>>>(rp, ci, va, xx, yy, n, st, scale, long_t); break;
    default: k_spmv<32, S><<<blocks, 256, 0, s>>>(rp, ci, va, xx, yy, n, st, scale, long_t); break;
  }
}

// ---- long rows: one warp per segment, then each long row merges its segment sums in order ----
__global__ void __launch_bounds__(256) k_spmv_seg_pair(LongRows lr, const float2 *__restrict__ va,
                                                       const int *__restrict__ ci, const float2 *__restrict__ x,
                                                       const KrylovState *st) {
  if (st && st->stop) return;
  const int lane = threadIdx.x & 31;
  const long long w0 = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
  unsigned long long *part = static_cast<unsigned long long *>(lr.part);
  for (long long sgi = w0; sgi < lr.n_seg; sgi += nw) {
    dfacc acc;
    acc_zero(acc);
    for (int p = lr.seg_beg[sgi] + lane; p < lr.seg_end[sgi]; p += 32) {
      const float2 av = __ldcs(va + p), xv = __ldg(x + __ldcs(ci + p));
      f2x a2, x2;
      a2.hi = av.x; a2.lo = av.y;
      x2.hi = xv.x; x2.lo = xv.y;
      acc_fma(acc, a2, x2);
    }
    acc = warp_reduce<PairAr>(acc);
    if (lane == 0) part[sgi] = PairAr::pack(acc);
  }
}

__global__ void k_spmv_longfix_pair(LongRows lr, float2 *__restrict__ y, const KrylovState *st, double scale) {
  if (st && st->stop) return;
  const f2x sc = split_f64(st ? st->sigma * scale : scale);
  const unsigned long long *part = static_cast<const unsigned long long *>(lr.part);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < lr.n_long; i += gridDim.x * blockDim.x) {
    dfacc acc;
    acc_zero(acc);
    for (int sgi = lr.lfirst[i]; sgi < lr.lfirst[i + 1]; ++sgi) acc_merge(acc, PairAr::unpack(part[sgi]));
    f2x v;
    v.hi = acc.s + acc.c;
    v.lo = acc.c - (v.hi - acc.s);
    dfacc pr;
    acc_zero(pr);
    acc_fma(pr, v, sc);
    const float hi = pr.s + pr.c;
    y[lr.lrow[i]] = make_float2(hi, pr.c - (hi - pr.s));
  }
}

__global__ void __launch_bounds__(256) k_spmv_seg_f32(LongRows lr, const float *__restrict__ va,
                                                      const int *__restrict__ ci, const float *__restrict__ x,
                                                      const KrylovState *st) {
  if (st && st->stop) return;
  const int lane = threadIdx.x & 31;
  const long long w0 = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
  unsigned long long *part = static_cast<unsigned long long *>(lr.part);
  for (long long sgi = w0; sgi < lr.n_seg; sgi += nw) {
    dfacc acc;
    acc_zero(acc);
    for (int p = lr.seg_beg[sgi] + lane; p < lr.seg_end[sgi]; p += 32) {
      f2x a2, x2;
      a2.hi = __ldcs(va + p);
      a2.lo = 0.0f;
      x2.hi = __ldg(x + __ldcs(ci + p));
      x2.lo = 0.0f;
      acc_fma(acc, a2, x2);
    }
    acc = warp_reduce<PairAr>(acc);
    if (lane == 0) part[sgi] = PairAr::pack(acc);
  }
}

__global__ void k_spmv_longfix_f32(LongRows lr, float *__restrict__ y, const KrylovState *st, double scale) {
  if (st && st->stop) return;
  const f2x sc = split_f64(st ? st->sigma * scale : scale);
  const unsigned long long *part = static_cast<const unsigned long long *>(lr.part);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < lr.n_long; i += gridDim.x * blockDim.x) {
    dfacc acc;
    acc_zero(acc);
    for (int sgi = lr.lfirst[i]; sgi < lr.lfirst[i + 1]; ++sgi) acc_merge(acc, PairAr::unpack(part[sgi]));
    f2x v;
    v.hi = acc.s + acc.c;
    v.lo = acc.c - (v.hi - acc.s);
    dfacc pr;
    acc_zero(pr);
    acc_fma(pr, v, sc);
    y[lr.lrow[i]] = pr.s + pr.c;
  }
}

__global__ void k_f64_to_f32(const double *x, float *y, long long n) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    y[i] = __double2float_rn(x[i]);
}

__global__ void k_f32_to_f64(const float *x, double *y, long long n) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    y[i] = (double)x[i];
}

template <class S>
__global__ void __launch_bounds__(256) k_spmv_seg_f64(LongRows lr, const double *__restrict__ va,
                                                      const int *__restrict__ ci, const typename S::T *__restrict__ x,
                                                      const KrylovState *st) {
  if (st && st->stop) return;
  const int lane = threadIdx.x & 31;
  const long long w0 = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
  double *part = static_cast<double *>(lr.part);
  for (long long sgi = w0; sgi < lr.n_seg; sgi += nw) {
    double sum = 0.0;
    for (int p = lr.seg_beg[sgi] + lane; p < lr.seg_end[sgi]; p += 32)
      sum = ::fma(__ldcs(va + p), S::get(x + __ldcs(ci + p)), sum);
    sum = warp_sum_f64(sum);
    if (lane == 0) part[sgi] = sum;
  }
}

template <class S>
__global__ void k_spmv_longfix_f64(LongRows lr, typename S::T *__restrict__ y, const KrylovState *st, double scale) {
  if (st && st->stop) return;
  const double sc = st ? st->sigma * scale : scale;
  const double *part = static_cast<const double *>(lr.part);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < lr.n_long; i += gridDim.x * blockDim.x) {
    double sum = 0.0;
    for (int sgi = lr.lfirst[i]; sgi < lr.lfirst[i + 1]; ++sgi) sum += part[sgi];
    S::put(y + lr.lrow[i], sum * sc);
  }
}

int spmv_blocks_for(int n, int lanes);
static int spmv_blocks(int n, int lanes) { return spmv_blocks_for(n, lanes); }

int restart_blocks_for(int n) {
  const int ntiles = (n + R_ROWS - 1) / R_ROWS;
  int blocks = num_sms();
  if (blocks > ntiles) blocks = ntiles;
  return blocks < 1 ? 1 : blocks;
}

int spmv_blocks_for(int n, int lanes) {
  const long long rows_per_block = (256 / 32) * (32 / lanes);
  long long blocks = (n + rows_per_block - 1) / rows_per_block;
  const long long cap = (long long)num_sms() * 16;
  if (blocks > cap) blocks = cap;
  return blocks < 1 ? 1 : (int)blocks;
}

cudaError_t launch_spmv(const int *rp, const int *ci, const double *va, const double *x, double *y, int n, int lanes,
                        const KrylovState *st, double scale, cudaStream_t s) {
  spmv_dispatch<StF64>(rp, ci, va, x, y, n, lanes, st, scale, spmv_blocks(n, lanes), s, 0x7fffffff);
  return cudaGetLastError();
}

cudaError_t launch_spmv_storage(const int *rp, const int *ci, const double *va, const float2 *va_pair, const void *x,
                                void *y, int n, int lanes, const KrylovState *st, double scale, int storage,
                                cudaStream_t s, const LongRows *lr, const float *va32) {
  const int blocks = spmv_blocks(n, lanes);
  const bool split = lr && lr->n_long > 0;
  const int long_t = split ? lr->long_t : 0x7fffffff;
  const int seg_blocks = split ? (int)std::min<long long>((lr->n_seg + 7) / 8, (long long)num_sms() * 8) : 0;
  if (storage == STORE_F32) {
    if (!va32) return cudaErrorInvalidValue;
    const float *xx = static_cast<const float *>(x);
    float *yy = static_cast<float *>(y);
    switch (lanes) {
      case 1: k_spmv_f32<1><<<blocks, 256, 0, s>>>(rp, ci, va32, xx, yy, n, st, scale, long_t); break;
      case 8: k_spmv_f32<8><<<blocks, 256, 0, s>>>(rp, ci, va32, xx, yy, n, st, scale, long_t); break;
      default: k_spmv_f32<32><<<blocks, 256, 0, s>>>(rp, ci, va32, xx, yy, n, st, scale, long_t); break;
    }
    if (split) {
      k_spmv_seg_f32<<<seg_blocks, 256, 0, s>>>(*lr, va32, ci, xx, st);
      k_spmv_longfix_f32<<<(lr->n_long + 127) / 128, 128, 0, s>>>(*lr, yy, st, scale);
    }
    return cudaGetLastError();
  }
  if (storage == STORE_F64) {
    spmv_dispatch<StF64>(rp, ci, va, x, y, n, lanes, st, scale, blocks, s, long_t);
    if (split) {
      k_spmv_seg_f64<StF64><<<seg_blocks, 256, 0, s>>>(*lr, va, ci, static_cast<const double *>(x), st);
      k_spmv_longfix_f64<StF64><<<(lr->n_long + 127) / 128, 128, 0, s>>>(*lr, static_cast<double *>(y), st, scale);
    }
  } else {
    const float2 *xx = static_cast<const float2 *>(x);
    float2 *yy = static_cast<float2 *>(y);
    switch (lanes) {
      case 1: k_spmv_pair<1><<<blocks, 256, 0, s>>>(rp, ci, va_pair, xx, yy, n, st, scale, long_t); break;
      case 2: k_spmv_pair<2><<<blocks, 256, 0, s>>>(rp, ci, va_pair, xx, yy, n, st, scale, long_t); break;
      case 4: k_spmv_pair<4><<<blocks, 256, 0, s>>>(rp, ci, va_pair, xx, yy, n, st, scale, long_t); break;
      case 8: k_spmv_pair<8><<<blocks, 256, 0, s>>>(rp, ci, va_pair, xx, yy, n, st, scale, long_t); break;
      case 16: k_spmv_pair<16><<<blocks, 256, 0, s>>>(rp, ci, va_pair, xx, yy, n, st, scale, long_t); break;
      default: k_spmv_pair<32><<<blocks, 256, 0, s>>>(rp, ci, va_pair, xx, yy, n, st, scale, long_t); break;
    }
    if (split) {
      k_spmv_seg_pair<<<seg_blocks, 256, 0, s>>>(*lr, va_pair, ci, xx, st);
      k_spmv_longfix_pair<<<(lr->n_long + 127) / 128, 128, 0, s>>>(*lr, yy, st, scale);
    }
  }
  return cudaGetLastError();
}

cudaError_t launch_f64_to_pair(const double *x, float2 *y, long long n, cudaStream_t s) {
  int blocks = (int)std::min<long long>((n + 255) / 256, (long long)num_sms() * 8);
  k_f64_to_pair<<<blocks < 1 ? 1 : blocks, 256, 0, s>>>(x, y, n);
  return cudaGetLastError();
}

cudaError_t launch_f64_to_f32(const double *x, float *y, long long n, cudaStream_t s) {
  int blocks = (int)std::min<long long>((n + 255) / 256, (long long)num_sms() * 8);
  k_f64_to_f32<<<blocks < 1 ? 1 : blocks, 256, 0, s>>>(x, y, n);
  return cudaGetLastError();
}

cudaError_t launch_f32_to_f64(const float *x, double *y, long long n, cudaStream_t s) {
  int blocks = (int)std::min<long long>((n + 255) / 256, (long long)num_sms() * 8);
  k_f32_to_f64<<<blocks < 1 ? 1 : blocks, 256, 0, s>>>(x, y, n);
  return cudaGetLastError();
}

cudaError_t launch_pair_to_f64(const float2 *x, double *y, long long n, cudaStream_t s) {
  int blocks = (int)std::min<long long>((n + 255) / 256, (long long)num_sms() * 8);
  k_pair_to_f64<<<blocks < 1 ? 1 : blocks, 256, 0, s>>>(x, y, n);
  return cudaGetLastError();
}

int gs_dot_blocks(int n) {
  const int ntiles = (n + A_TILE - 1) / A_TILE;
  int blocks = num_sms();
  if (blocks > ntiles) blocks = ntiles;
  return blocks < 1 ? 1 : blocks;
}

int gs_update_blocks(int n) {
  const int ntiles = (n + B_TILE - 1) / B_TILE;
  int blocks = num_sms() * 2;  // two resident blocks per SM at ~120 registers per thread; persistent over tiles
  if (blocks > ntiles) blocks = ntiles;
  return blocks < 1 ? 1 : blocks;
}

int gs_max_columns() { return A_MAXJ; }
int gs_wide_max_columns() { return GW_MAXJ; }
int restart_wide_max_columns() { return RW_MAXK; }

template <int NX, class Ar, class S>
static cudaError_t dot_dispatch(const StepArgs &a, int mode, int blocks, cudaStream_t s) {
  const int J = a.J;
  if (J <= 16) k_gs_dot<NX, 1, Ar, S><<<blocks, A_THREADS, 0, s>>>(a, mode);
  else if (J <= 32) k_gs_dot<NX, 2, Ar, S><<<blocks, A_THREADS, 0, s>>>(a, mode);
  else if (J <= 64) k_gs_dot<NX, 4, Ar, S><<<blocks, A_THREADS, 0, s>>>(a, mode);
  else if (J <= 144) k_gs_dot<NX, 9, Ar, S><<<blocks, A_THREADS, 0, s>>>(a, mode);
  else if (J <= A_MAXJ) k_gs_dot<NX, 17, Ar, S><<<blocks, A_THREADS, 0, s>>>(a, mode);
  else if (J <= GW_MAXJ) k_gs_dot_wide<NX, Ar, S><<<blocks, A_THREADS, (size_t)(2 * J + 4) * 8, s>>>(a, mode);
  else return cudaErrorInvalidValue;
  return cudaGetLastError();
}

// storage: STORE_F64 (doubles) or STORE_PAIR (FP32 pairs, pair arithmetic only)
// the exact-product pair (tensor cores or integer pipes) runs IEEE-double Gram-Schmidt when the caller supplies its
// arguments and the basis has columns
static bool gs_use_tc(const StepArgs &a, int arith, int storage) {
  return a.tc && storage == STORE_F64 && arith == ARITH_F64 && a.J >= 1 && a.J <= gs_tc_max_columns();
}

cudaError_t launch_gs_dot(const StepArgs &a, int nx, int mode, int arith, cudaStream_t s, int storage,
                          int max_blocks) {
  if (gs_use_tc(a, arith, storage))
    return a.tc->integer ? launch_gs_dot_ix(a, nx, mode, *a.tc, s) : launch_gs_dot_tc(a, nx, mode, *a.tc, s);
  int blocks = gs_dot_blocks(a.n);
  if (max_blocks > 0 && blocks > max_blocks) blocks = max_blocks;
  if (storage == STORE_F32)
    return nx == 2 ? dot_dispatch<2, PairAr, StF32>(a, mode, blocks, s) : dot_dispatch<1, PairAr, StF32>(a, mode, blocks, s);
  if (storage == STORE_PAIR)
    return nx == 2 ? dot_dispatch<2, PairAr, StPair>(a, mode, blocks, s) : dot_dispatch<1, PairAr, StPair>(a, mode, blocks, s);
  if (arith == ARITH_F64)
    return nx == 2 ? dot_dispatch<2, F64Ar, StF64>(a, mode, blocks, s) : dot_dispatch<1, F64Ar, StF64>(a, mode, blocks, s);
  return nx == 2 ? dot_dispatch<2, PairAr, StF64>(a, mode, blocks, s) : dot_dispatch<1, PairAr, StF64>(a, mode, blocks, s);
}

cudaError_t launch_gs_update(const StepArgs &a, int nx, int mode, int arith, cudaStream_t s, int storage) {
  if (gs_use_tc(a, arith, storage))
    return a.tc->integer ? launch_gs_update_ix(a, nx, mode, *a.tc, s) : launch_gs_update_tc(a, nx, mode, *a.tc, s);
  if (a.tc && storage == STORE_F64 && arith == ARITH_F64 && mode != GS_COMBINE) {
    // the FP64-FMA kernel writes the column (no basis columns to project out): record its tile exponents for the
    // tensor-core launches that read it later
    StepArgs b = a;
    b.tc = nullptr;
    const cudaError_t e = launch_gs_update(b, nx, mode, arith, s, storage);
    if (e != cudaSuccess) return e;
    return launch_record_vexp(static_cast<const double *>(a.U), a.n, a.tc->vexp + (size_t)a.j * a.tc->ldt, s);
  }
  const int blocks = gs_update_blocks(a.n);
  const size_t shm = (size_t)nx * (a.J > 0 ? a.J : 1) * 8;
  if (storage == STORE_F32) {
    if (nx == 2) k_gs_update<2, PairAr, StF32><<<blocks, B_THREADS, shm, s>>>(a, mode);
    else k_gs_update<1, PairAr, StF32><<<blocks, B_THREADS, shm, s>>>(a, mode);
  } else if (storage == STORE_PAIR) {
    if (nx == 2) k_gs_update<2, PairAr, StPair><<<blocks, B_THREADS, shm, s>>>(a, mode);
    else k_gs_update<1, PairAr, StPair><<<blocks, B_THREADS, shm, s>>>(a, mode);
  } else if (arith == ARITH_F64) {
    if (nx == 2) k_gs_update<2, F64Ar, StF64><<<blocks, B_THREADS, shm, s>>>(a, mode);
    else k_gs_update<1, F64Ar, StF64><<<blocks, B_THREADS, shm, s>>>(a, mode);
  } else {
    if (nx == 2) k_gs_update<2, PairAr, StF64><<<blocks, B_THREADS, shm, s>>>(a, mode);
    else k_gs_update<1, PairAr, StF64><<<blocks, B_THREADS, shm, s>>>(a, mode);
  }
  return cudaGetLastError();
}

size_t restart_smem_bytes(int K, int N, int tile_rows) { return ((size_t)K * N + (size_t)K * tile_rows) * 8; }

// one restart launch with CQ column chunks (N <= 16 CQ)
template <class Ar, class S, int CQ>
static cudaError_t restart_go(typename S::T *V, long long ldv, int n, int a0, int K, int s0, int N, const double *Q,
                              int ldq, cudaStream_t s) {
  constexpr int TR = restart_tile_rows<CQ>();
  const size_t shm = restart_smem_bytes(K, N, TR);
  if (shm > 227 * 1024) return cudaErrorInvalidValue;
  const int ntiles = (n + TR - 1) / TR;
  // two resident blocks per SM when shared memory allows
  const int per_sm = shm * 2 <= (size_t)227 * 1024 ? 2 : 1;
  int blocks = num_sms() * per_sm;
  if (blocks > ntiles) blocks = ntiles;
  const cudaError_t err = cudaFuncSetAttribute(k_restart<Ar, S, CQ>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm);
  if (err != cudaSuccess) return err;
  k_restart<Ar, S, CQ><<<blocks, R_THREADS, shm, s>>>(V, ldv, n, a0, K, s0, N, Q, ldq);
  return cudaGetLastError();
}

template <class Ar, class S>
static cudaError_t restart_wide_go(typename S::T *V, long long ldv, int n, int a0, int K, int s0, int N,
                                   const double *Q, int ldq, cudaStream_t s) {
  if (K > RW_MAXK) return cudaErrorInvalidValue;
  const size_t shm = (size_t)K * RW_ROWS * sizeof(typename Ar::val);
  const int ntiles = (n + RW_ROWS - 1) / RW_ROWS;
  int blocks = num_sms() * (shm * 2 <= (size_t)227 * 1024 ? 2 : 1);
  if (blocks > ntiles) blocks = ntiles;
  const cudaError_t err = cudaFuncSetAttribute(k_restart_wide<Ar, S>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                               (int)shm);
  if (err != cudaSuccess) return err;
  k_restart_wide<Ar, S><<<blocks, R_THREADS, shm, s>>>(V, ldv, n, a0, K, s0, N, Q, ldq);
  return cudaGetLastError();
}

template <class Ar, class S>
static cudaError_t restart_dispatch(typename S::T *V, long long ldv, int n, int a0, int K, int s0, int N,
                                    const double *Q, int ldq, cudaStream_t s) {
  if (K > R_MAXN || N > R_MAXN) return restart_wide_go<Ar, S>(V, ldv, n, a0, K, s0, N, Q, ldq, s);
  if (N <= 16) return restart_go<Ar, S, 1>(V, ldv, n, a0, K, s0, N, Q, ldq, s);
  if (N <= 32) return restart_go<Ar, S, 2>(V, ldv, n, a0, K, s0, N, Q, ldq, s);
  if (N <= 64) return restart_go<Ar, S, 4>(V, ldv, n, a0, K, s0, N, Q, ldq, s);
  return restart_go<Ar, S, 9>(V, ldv, n, a0, K, s0, N, Q, ldq, s);
}

cudaError_t launch_restart(void *V, long long ldv, int n, int a0, int K, int s0, int N, const double *Q, int ldq,
                           int arith, cudaStream_t s, int storage) {
  if (N <= 0 || K <= 0) return cudaSuccess;
  if (N > RW_MAXK || K > RW_MAXK) return cudaErrorInvalidValue;
  if (storage == STORE_F32)
    return restart_dispatch<PairAr, StF32>(static_cast<float *>(V), ldv, n, a0, K, s0, N, Q, ldq, s);
  if (storage == STORE_PAIR)
    return restart_dispatch<PairAr, StPair>(static_cast<float2 *>(V), ldv, n, a0, K, s0, N, Q, ldq, s);
  if (arith == ARITH_F64)
    return restart_dispatch<F64Ar, StF64>(static_cast<double *>(V), ldv, n, a0, K, s0, N, Q, ldq, s);
  return restart_dispatch<PairAr, StF64>(static_cast<double *>(V), ldv, n, a0, K, s0, N, Q, ldq, s);
}

cudaError_t launch_segment_begin(KrylovState *st, int k0, int m, cudaStream_t s) {
  k_segment_begin<<<1, 1, 0, s>>>(st, k0, m);
  return cudaGetLastError();
}

cudaError_t launch_set_scales(KrylovState *st, double sigma, double invnu, cudaStream_t s) {
  k_set_scales<<<1, 1, 0, s>>>(st, sigma, invnu);
  return cudaGetLastError();
}

cudaError_t launch_set_unit_scale(KrylovState *st, cudaStream_t s) { return launch_set_scales(st, 1.0, 1.0, s); }

cudaError_t launch_negate(void *x, long long count, int as_float, cudaStream_t s) {
  int blocks = (int)std::min<long long>((count + 255) / 256, (long long)num_sms() * 8);
  if (blocks < 1) blocks = 1;
  if (as_float) k_negate_f32<<<blocks, 256, 0, s>>>(static_cast<float *>(x), count);
  else k_negate<<<blocks, 256, 0, s>>>(static_cast<double *>(x), count);
  return cudaGetLastError();
}

cudaError_t launch_scale(double *x, int n, double alpha, cudaStream_t s) {
  int blocks = (n + 255) / 256;
  if (blocks > num_sms() * 8) blocks = num_sms() * 8;
  if (blocks < 1) blocks = 1;
  k_scale_col<<<blocks, 256, 0, s>>>(x, n, alpha);
  return cudaGetLastError();
}

}  // namespace ksg
