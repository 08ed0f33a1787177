// krylov_body.cuh -- arithmetic/storage traits and the device bodies of the Krylov factorisation kernels.
//
// Each body takes the index of its block and the number of blocks taking part (bid, nblk) instead of reading
// blockIdx/gridDim, so the same code runs as a whole-grid kernel for one problem (k_krylov.cu) and as the share
// of one instance inside a batched launch (k_batch.cu).  The per-instance arithmetic -- and so every rounding --
// is identical in both.
#pragma once

#include "common.cuh"
#include "ks_types.h"

namespace ksg {

// ------------------------------------------------------------------------------------------------------------
// Arithmetic traits
// ------------------------------------------------------------------------------------------------------------
struct PairAr {
  using val = f2x;
  using acc = dfacc;
  static KS_DEVICE val cvt(double v) { return split_f64(v); }
  static KS_DEVICE void zero(acc &a) { acc_zero(a); }
  static KS_DEVICE void fma(acc &a, val x, val y) { acc_fma(a, x, y); }
  static KS_DEVICE void merge(acc &a, acc b) { acc_merge(a, b); }
  static KS_DEVICE double value(acc a) { return acc_value(a); }
  static KS_DEVICE acc shfl(acc a, int off) { return shfl_down_acc(a, off); }
  static KS_DEVICE unsigned long long pack(acc a) {
    return (unsigned long long)__float_as_uint(a.s) | ((unsigned long long)__float_as_uint(a.c) << 32);
  }
  static KS_DEVICE acc unpack(unsigned long long u) {
    acc a;
    a.s = __uint_as_float((unsigned)(u & 0xffffffffull));
    a.c = __uint_as_float((unsigned)(u >> 32));
    return a;
  }
};

struct F64Ar {
  using val = double;
  using acc = double;
  static KS_DEVICE val cvt(double v) { return v; }
  static KS_DEVICE void zero(acc &a) { a = 0.0; }
  static KS_DEVICE void fma(acc &a, val x, val y) { a = ::fma(x, y, a); }
  static KS_DEVICE void merge(acc &a, acc b) { a += b; }
  static KS_DEVICE double value(acc a) { return a; }
  static KS_DEVICE acc shfl(acc a, int off) { return __shfl_down_sync(0xffffffffu, a, off); }
  static KS_DEVICE unsigned long long pack(acc a) { return (unsigned long long)__double_as_longlong(a); }
  static KS_DEVICE acc unpack(unsigned long long u) { return __longlong_as_double((long long)u); }
};

// ------------------------------------------------------------------------------------------------------------
// Basis storage formats.  StF64: IEEE doubles.  StPair: FP32 pairs (hi, lo) with hi + lo the stored value (47-bit
// significand, the same 8 bytes per entry), so the pair arithmetic reads them without any conversion.
// load2 reads entries i and i+1 (i even, 16-byte aligned) in one vector load that bypasses L1 residency.
// ------------------------------------------------------------------------------------------------------------
struct StF64 {
  using T = double;
  template <class Ar>
  static KS_DEVICE void load2(const T *p, typename Ar::val &a, typename Ar::val &b) {
    const double2 v = __ldcs(reinterpret_cast<const double2 *>(p));
    a = Ar::cvt(v.x);
    b = Ar::cvt(v.y);
  }
  template <class Ar>
  static KS_DEVICE typename Ar::val load1(const T *p) { return Ar::cvt(*p); }
  static KS_DEVICE double get(const T *p) { return *p; }
  static KS_DEVICE void put(T *p, double v) { *p = v; }
  static KS_DEVICE void get2(const T *p, double &a, double &b) {
    const double2 v = *reinterpret_cast<const double2 *>(p);
    a = v.x;
    b = v.y;
  }
  static KS_DEVICE void put2(T *p, double a, double b) { *reinterpret_cast<double2 *>(p) = make_double2(a, b); }
};

struct StPair {
  using T = float2;
  template <class Ar>
  static KS_DEVICE void load2(const T *p, typename Ar::val &a, typename Ar::val &b) {
    const float4 v = __ldcs(reinterpret_cast<const float4 *>(p));
    a = pair_val<Ar>(v.x, v.y);
    b = pair_val<Ar>(v.z, v.w);
  }
  template <class Ar>
  static KS_DEVICE typename Ar::val load1(const T *p) {
    const float2 v = *p;
    return pair_val<Ar>(v.x, v.y);
  }
  template <class Ar>
  static KS_DEVICE typename Ar::val pair_val(float hi, float lo);
  static KS_DEVICE double get(const T *p) {
    const float2 v = *p;
    return (double)v.x + (double)v.y;
  }
  static KS_DEVICE void put(T *p, double v) {
    const f2x s = split_f64(v);
    *p = make_float2(s.hi, s.lo);
  }
  static KS_DEVICE void get2(const T *p, double &a, double &b) {
    const float4 v = *reinterpret_cast<const float4 *>(p);
    a = (double)v.x + (double)v.y;
    b = (double)v.z + (double)v.w;
  }
  static KS_DEVICE void put2(T *p, double a, double b) {
    const f2x x = split_f64(a), y = split_f64(b);
    *reinterpret_cast<float4 *>(p) = make_float4(x.hi, x.lo, y.hi, y.lo);
  }
};
template <>
KS_DEVICE PairAr::val StPair::pair_val<PairAr>(float hi, float lo) {
  f2x r;
  r.hi = hi;
  r.lo = lo;
  return r;
}
template <>
KS_DEVICE F64Ar::val StPair::pair_val<F64Ar>(float hi, float lo) {
  return (double)hi + (double)lo;
}

// StF32: FP32 entries (the precision form: half the bytes of the other formats).  Values widen exactly into the
// pair arithmetic, so every product and sum is still accumulated at FP64-class accuracy; only storage rounds.
struct StF32 {
  using T = float;
  template <class Ar>
  static KS_DEVICE typename Ar::val widen(float v);
  template <class Ar>
  static KS_DEVICE void load2(const T *p, typename Ar::val &a, typename Ar::val &b) {
    const float2 v = __ldcs(reinterpret_cast<const float2 *>(p));
    a = widen<Ar>(v.x);
    b = widen<Ar>(v.y);
  }
  template <class Ar>
  static KS_DEVICE typename Ar::val load1(const T *p) { return widen<Ar>(*p); }
  static KS_DEVICE double get(const T *p) { return (double)*p; }
  static KS_DEVICE void put(T *p, double v) { *p = __double2float_rn(v); }
  static KS_DEVICE void get2(const T *p, double &a, double &b) {
    const float2 v = *reinterpret_cast<const float2 *>(p);
    a = (double)v.x;
    b = (double)v.y;
  }
  static KS_DEVICE void put2(T *p, double a, double b) {
    *reinterpret_cast<float2 *>(p) = make_float2(__double2float_rn(a), __double2float_rn(b));
  }
};
template <>
KS_DEVICE PairAr::val StF32::widen<PairAr>(float v) {
  f2x r;
  r.hi = v;
  r.lo = 0.0f;
  return r;
}
template <>
KS_DEVICE F64Ar::val StF32::widen<F64Ar>(float v) {
  return (double)v;
}

template <class Ar>
KS_DEVICE typename Ar::acc warp_reduce(typename Ar::acc a) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) Ar::merge(a, Ar::shfl(a, off));
  return a;
}

KS_DEVICE double warp_sum_f64(double v) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
  return v;
}

enum { TK_DOT = 0, TK_UPD = 1, TK_NRM = 2 };

// ------------------------------------------------------------------------------------------------------------
// SpMV: LANES threads per row, FP64 FMA.  Each warp owns 32/LANES consecutive rows per iteration.
// ------------------------------------------------------------------------------------------------------------
// Rows with more than long_t nonzeros are skipped: the segment kernels of k_krylov.cu compute them.
template <int LANES, class S>
__global__ void __launch_bounds__(256) k_spmv(const int *__restrict__ rp, const int *__restrict__ ci,
                                              const double *__restrict__ va, const typename S::T *__restrict__ x,
                                              typename S::T *__restrict__ y, int n, const KrylovState *st,
                                              double scale, int long_t) {
  if (st && st->stop) return;
  const double sc = st ? st->sigma * scale : scale;
  constexpr int RPW = 32 / LANES;
  const int lane = threadIdx.x & 31;
  const int sub = lane % LANES, grp = lane / LANES;
  const long long warp_global = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
  for (long long base = warp_global * RPW; base < n; base += nwarps * RPW) {
    const long long row = base + grp;
    int p0 = 0, p1 = 0;
    bool seg = false;  // a long row: computed by the segment kernels
    if (row < n) {
      p0 = rp[row];
      p1 = rp[row + 1];
      if (p1 - p0 > long_t) {
        seg = true;
        p1 = p0;
      }
    }
    double sum = 0.0;
    for (int p = p0 + sub; p < p1; p += LANES) sum = ::fma(__ldcs(va + p), S::get(x + __ldcs(ci + p)), sum);
#pragma unroll
    for (int off = LANES / 2; off > 0; off >>= 1) sum += __shfl_down_sync(0xffffffffu, sum, off, LANES);
    if (sub == 0 && row < n && !seg) S::put(y + row, sum * sc);
  }
}

// SpMV for pair storage: matrix values pre-split into pairs, x gathered as pairs, products and sums in pair
// arithmetic, the scale applied as a pair product; nothing touches the FP64 pipe.
// The rows handled by warp `warp_global` of `nwarps` (a kernel's whole grid, or the virtual blocks one instance of
// a batch owns).
template <int LANES>
KS_DEVICE void spmv_pair_rows(const int *__restrict__ rp, const int *__restrict__ ci, const float2 *__restrict__ va,
                              const float2 *__restrict__ x, float2 *__restrict__ y, int n, const KrylovState *st,
                              double scale, long long warp_global, long long nwarps, int long_t = 0x7fffffff) {
  if (st && st->stop) return;
  const f2x sc = split_f64(st ? st->sigma * scale : scale);
  constexpr int RPW = 32 / LANES;
  const int lane = threadIdx.x & 31;
  const int sub = lane % LANES, grp = lane / LANES;
  for (long long base = warp_global * RPW; base < n; base += nwarps * RPW) {
    const long long row = base + grp;
    int p0 = 0, p1 = 0;
    bool seg = false;  // a long row: computed by the segment kernels
    if (row < n) {
      p0 = rp[row];
      p1 = rp[row + 1];
      if (p1 - p0 > long_t) {
        seg = true;
        p1 = p0;
      }
    }
    dfacc acc;
    acc_zero(acc);
    for (int p = p0 + sub; p < p1; p += LANES) {
      // the matrix streams through once per step (evict-first); the gathered x stays in L2
      const float2 av = __ldcs(va + p), xv = __ldg(x + __ldcs(ci + p));
      f2x a2, x2;
      a2.hi = av.x; a2.lo = av.y;
      x2.hi = xv.x; x2.lo = xv.y;
      acc_fma(acc, a2, x2);
    }
#pragma unroll
    for (int off = LANES / 2; off > 0; off >>= 1) {
      dfacc o;
      o.s = __shfl_down_sync(0xffffffffu, acc.s, off, LANES);
      o.c = __shfl_down_sync(0xffffffffu, acc.c, off, LANES);
      acc_merge(acc, o);
    }
    if (sub == 0 && row < n && !seg) {
      // renormalise (s, c) into a pair, then multiply by the scale as pairs
      f2x v;
      v.hi = acc.s + acc.c;
      v.lo = acc.c - (v.hi - acc.s);
      dfacc pr;
      acc_zero(pr);
      acc_fma(pr, v, sc);
      const float hi = pr.s + pr.c;
      y[row] = make_float2(hi, pr.c - (hi - pr.s));
    }
  }
}

// SpMV of the precision form: FP32 values and vectors, products exact in pairs, pair accumulation, result rounded
// to FP32 once.
template <int LANES>
KS_DEVICE void spmv_f32_rows(const int *__restrict__ rp, const int *__restrict__ ci, const float *__restrict__ va,
                             const float *__restrict__ x, float *__restrict__ y, int n, const KrylovState *st,
                             double scale, long long warp_global, long long nwarps, int long_t = 0x7fffffff) {
  if (st && st->stop) return;
  const f2x sc = split_f64(st ? st->sigma * scale : scale);
  constexpr int RPW = 32 / LANES;
  const int lane = threadIdx.x & 31;
  const int sub = lane % LANES, grp = lane / LANES;
  for (long long base = warp_global * RPW; base < n; base += nwarps * RPW) {
    const long long row = base + grp;
    int p0 = 0, p1 = 0;
    bool seg = false;
    if (row < n) {
      p0 = rp[row];
      p1 = rp[row + 1];
      if (p1 - p0 > long_t) {
        seg = true;
        p1 = p0;
      }
    }
    dfacc acc;
    acc_zero(acc);
    for (int p = p0 + sub; p < p1; p += LANES) {
      f2x a2, x2;
      a2.hi = __ldcs(va + p);
      a2.lo = 0.0f;
      x2.hi = __ldg(x + __ldcs(ci + p));
      x2.lo = 0.0f;
      acc_fma(acc, a2, x2);
    }
#pragma unroll
    for (int off = LANES / 2; off > 0; off >>= 1) {
      dfacc o;
      o.s = __shfl_down_sync(0xffffffffu, acc.s, off, LANES);
      o.c = __shfl_down_sync(0xffffffffu, acc.c, off, LANES);
      acc_merge(acc, o);
    }
    if (sub == 0 && row < n && !seg) {
      f2x v;
      v.hi = acc.s + acc.c;
      v.lo = acc.c - (v.hi - acc.s);
      dfacc pr;
      acc_zero(pr);
      acc_fma(pr, v, sc);
      y[row] = pr.s + pr.c;
    }
  }
}

template <int LANES>
__global__ void __launch_bounds__(256) k_spmv_f32(const int *__restrict__ rp, const int *__restrict__ ci,
                                                  const float *__restrict__ va, const float *__restrict__ x,
                                                  float *__restrict__ y, int n, const KrylovState *st, double scale,
                                                  int long_t) {
  spmv_f32_rows<LANES>(rp, ci, va, x, y, n, st, scale, ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5,
                       ((long long)gridDim.x * blockDim.x) >> 5, long_t);
}

template <int LANES>
__global__ void __launch_bounds__(256) k_spmv_pair(const int *__restrict__ rp, const int *__restrict__ ci,
                                                   const float2 *__restrict__ va, const float2 *__restrict__ x,
                                                   float2 *__restrict__ y, int n, const KrylovState *st,
                                                   double scale, int long_t) {
  spmv_pair_rows<LANES>(rp, ci, va, x, y, n, st, scale, ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5,
                        ((long long)gridDim.x * blockDim.x) >> 5, long_t);
}

// ------------------------------------------------------------------------------------------------------------
// Gram-Schmidt half A: partial sums of V^T u (and V^T w), plus u.u (u.w, w.w), per block, then the last block
// merges them in block order and runs the coefficient algebra (epilogues below).
// ------------------------------------------------------------------------------------------------------------
constexpr int A_THREADS = 512;
constexpr int A_WARPS = 16;
constexpr int A_TILE = 512;
constexpr int A_MAXJ = 272;

// Coefficient algebra of one DCGS2 step (mode 0), the final reorthogonalisation (mode 1) or a plain CGS pass
// used to orthonormalise a start vector (mode 2).  res[] holds the merged sums: s_raw/b interleaved per column
// (NX = 2) or s_raw only (NX = 1), then the scalars.  Runs in the last block.
template <int NX>
__device__ void gs_epilogue(const StepArgs &a, const double *res, int mode) {
  KrylovState *st = a.st;
  // res[] already carries the scale sigma: kernel A stages u = sigma * u_raw
  if (mode == GS_DOTS) {
    for (int i = threadIdx.x; i < a.J * NX; i += blockDim.x) a.coef[i] = res[i];
    if (threadIdx.x == 0) a.coef[a.J * NX] = res[a.J * NX];
    return;
  }
  const int J = a.J, j = a.j;
  const int off = a.nc;  // coefficient of Krylov column i: coef[off + i] (constraint columns come first)
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  __shared__ double sh_nu, sh_bp, sh_tau, sh_invnu, sh_hj, sh_sigma;
  __shared__ int sh_lindep, sh_first;
  const double sigma = st->sigma;
  if (warp == 0) {
    double ss = 0.0, sb = 0.0;
    for (int i = lane; i < J; i += 32) {
      const double s = res[i * NX];
      ss = ::fma(s, s, ss);
      if (NX == 2) sb = ::fma(s, res[i * NX + 1], sb);
      a.coef[i] = s;
    }
    ss = warp_sum_f64(ss);
    sb = warp_sum_f64(sb);
    if (lane == 0) {
      const double aa = res[J * NX];
      const double nu2 = aa - ss;
      const double onorm = sqrt(aa > 0.0 ? aa : 0.0);
      const double nu = nu2 > 0.0 ? sqrt(nu2) : 0.0;
      // a column orthogonalised against n columns (a full basis) is zero: breakdown with beta = 0, as the
      // reference's safe orthogonalisation of the last column (bvkrylov.c:90, bvimpl.h:452-465)
      const int full = J >= a.n && mode != 2;
      const int lindep = full || !(nu2 > 0.0 && nu >= a.eta * onorm);
      sh_nu = nu;
      sh_lindep = lindep;
      sh_sigma = sigma;
      sh_bp = st->beta_prev;
      sh_first = (j == st->k0) || mode == 2;
      st->onorm = onorm;
      if (mode == 2) {
        // one CGS pass of an orthonormalisation: the caller judges linear dependence from nu and onorm
        st->breakdown = !(nu2 > 0.0 && nu > 0.0);
        if (!st->breakdown) st->invnu = 1.0 / nu;
        else st->stop = 1;
      } else if (lindep) {
        st->stop = 1;
        st->breakdown = 1;
        if (mode == 0) st->m = j;
        st->beta_out = full ? 0.0 : st->beta_prev * nu;
      } else {
        const double invnu = 1.0 / nu;
        sh_invnu = invnu;
        st->invnu = invnu;
        if (mode == 1) {
          st->beta_out = st->beta_prev * nu;
        } else {
          const double c = res[J * NX + 1];
          const double hj = (c - sb) * invnu;
          const double tau = hj * invnu;
          sh_hj = hj;
          sh_tau = tau;
          st->tau_sigma = tau * sigma;
        }
      }
    }
  }
  __syncthreads();
  if (mode == 2) return;
  const int lindep = sh_lindep, first = sh_first;
  const double bp = sh_bp, nu = sh_nu;
  // 1. finalise column j-1 (columns of this segment only): H[0:j, j-1] += bp * s, H[j, j-1] = bp * nu
  if (!first) {
    if (a.hermitian) {
      if (tid == 0) {
        a.d[j - 1] += bp * a.coef[off + j - 1];
        a.e[j - 1] = lindep ? 0.0 : bp * nu;
      }
    } else {
      for (int i = tid; i < j; i += blockDim.x) a.H[i + (size_t)(j - 1) * a.ldh] += bp * a.coef[off + i];
      if (tid == 0) a.H[j + (size_t)(j - 1) * a.ldh] = lindep ? 0.0 : bp * nu;
    }
  }
  if (mode == 1 || lindep) return;
  __syncthreads();
  // 2. column j: H[0:j+1, j] = ([b; hj] - H[0:j+1, 0:j] s) / nu;  g = b - tau s
  const double invnu = sh_invnu, tau = sh_tau, hj = sh_hj;
  if (a.hermitian) {
    if (warp == 0) {
      // row j of H[0:j+1, 0:j]: the arrow (first step of a segment) or the subdiagonal entry
      double hs = 0.0;
      if (first) {
        for (int i = lane; i < j; i += 32) hs = ::fma(a.e[i], a.coef[off + i], hs);
        hs = warp_sum_f64(hs);
      } else if (lane == 0) {
        hs = a.e[j - 1] * a.coef[off + j - 1];
      }
      if (lane == 0) a.d[j] = (hj - hs) * invnu;
    }
  } else {
    double *Hc = a.H + (size_t)j * a.ldh;
    for (int i = tid; i <= j; i += blockDim.x) {
      double hs = 0.0;
      const int c0 = (i >= 2) ? 0 : 0;
      for (int c = c0; c < j; ++c) hs = ::fma(a.H[i + (size_t)c * a.ldh], a.coef[off + c], hs);
      const double y = (i < j) ? res[(off + i) * NX + 1] : hj;
      Hc[i] = (y - hs) * invnu;
    }
  }
  for (int i = tid; i < J; i += blockDim.x) a.coef[J + i] = res[i * NX + 1] - tau * a.coef[i];
}

// Block `bid` of `nblk` taking part in one instance's reduction (bid/nblk are the grid's own for a single problem).
template <int NX, int CPW, class Ar, class S>
KS_DEVICE void gs_dot_body(const StepArgs &a, int mode, int bid, int nblk) {
  KrylovState *st = a.st;
  if (st->stop) return;
  using val = typename Ar::val;
  using acc = typename Ar::acc;
  __shared__ __align__(16) val sx[NX][A_TILE];
  __shared__ acc sred[A_WARPS][3];
  __shared__ double res[A_MAXJ * 2 + 4];
  __shared__ int s_last;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int n = a.n, J = a.J;
  const double sigma = st->sigma;
  using ST = typename S::T;
  const ST *Vb = static_cast<const ST *>(a.V);
  const ST *U = static_cast<const ST *>(a.U);
  const ST *W = static_cast<const ST *>(a.W);
  acc cacc[CPW][NX];
#pragma unroll
  for (int k = 0; k < CPW; ++k)
#pragma unroll
    for (int q = 0; q < NX; ++q) Ar::zero(cacc[k][q]);
  acc sc0, sc1, sc2;
  Ar::zero(sc0);
  Ar::zero(sc1);
  Ar::zero(sc2);
  const int ntiles = (n + A_TILE - 1) / A_TILE;
  val na[8], nb[8];
  bool have_next = false;
  for (int t = bid; t < ntiles; t += nblk) {
    const int r0 = t * A_TILE;
    const int rows = min(A_TILE, n - r0);
    {
      double u = 0.0, w = 0.0;
      if (tid < rows) {
        u = S::get(U + r0 + tid) * sigma;
        if (NX == 2) w = S::get(W + r0 + tid);
      }
      const val us = Ar::cvt(u);
      sx[0][tid] = us;
      Ar::fma(sc0, us, us);
      if (NX == 2) {
        const val ws = Ar::cvt(w);
        sx[NX - 1][tid] = ws;
        Ar::fma(sc1, us, ws);
        Ar::fma(sc2, ws, ws);
      }
    }
    __syncthreads();
    if (rows == A_TILE) {
      // software pipeline: the column of the next (k+1) iteration -- or the first column of this warp in the
      // block's next tile -- is loaded before the current column is consumed
      if (!have_next && warp < J) {
        const ST *col = Vb + (size_t)warp * a.ldv + r0 + lane * 2;
#pragma unroll
        for (int i = 0; i < 8; ++i) S::template load2<Ar>(col + 64 * i, na[i], nb[i]);
      }
      have_next = false;
#pragma unroll
      for (int k = 0; k < CPW; ++k) {
        const int c = warp + k * A_WARPS;
        if (c < J) {
          val ca[8], cb[8];
#pragma unroll
          for (int i = 0; i < 8; ++i) {
            ca[i] = na[i];
            cb[i] = nb[i];
          }
          int cn = c + A_WARPS, tn = t;
          if (cn >= J) {
            cn = warp;
            tn = t + nblk;
          }
          if (tn < ntiles && (tn + 1) * A_TILE <= n) {
            const ST *col = Vb + (size_t)cn * a.ldv + (size_t)tn * A_TILE + lane * 2;
#pragma unroll
            for (int i = 0; i < 8; ++i) S::template load2<Ar>(col + 64 * i, na[i], nb[i]);
            if (tn != t) have_next = true;
          }
#pragma unroll
          for (int i = 0; i < 8; ++i) {
            const int rr = lane * 2 + 64 * i;
            Ar::fma(cacc[k][0], ca[i], sx[0][rr]);
            Ar::fma(cacc[k][0], cb[i], sx[0][rr + 1]);
            if (NX == 2) {
              Ar::fma(cacc[k][NX - 1], ca[i], sx[NX - 1][rr]);
              Ar::fma(cacc[k][NX - 1], cb[i], sx[NX - 1][rr + 1]);
            }
          }
        }
      }
    } else {
#pragma unroll
      for (int k = 0; k < CPW; ++k) {
        const int c = warp + k * A_WARPS;
        if (c < J) {
          const ST *col = Vb + (size_t)c * a.ldv + r0;
          for (int rr = lane; rr < rows; rr += 32) {
            const val a0 = S::template load1<Ar>(col + rr);
            Ar::fma(cacc[k][0], a0, sx[0][rr]);
            if (NX == 2) Ar::fma(cacc[k][NX - 1], a0, sx[NX - 1][rr]);
          }
        }
      }
    }
    __syncthreads();
  }
  // per-block partials
  unsigned long long *pb = reinterpret_cast<unsigned long long *>(a.part) + (size_t)bid * a.pstride;
#pragma unroll
  for (int k = 0; k < CPW; ++k) {
    const int c = warp + k * A_WARPS;
    if (c < J) {
#pragma unroll
      for (int q = 0; q < NX; ++q) {
        const acc r = warp_reduce<Ar>(cacc[k][q]);
        if (lane == 0) pb[c * NX + q] = Ar::pack(r);
      }
    }
  }
  {
    acc r0 = warp_reduce<Ar>(sc0), r1 = warp_reduce<Ar>(sc1), r2 = warp_reduce<Ar>(sc2);
    if (lane == 0) {
      sred[warp][0] = r0;
      sred[warp][1] = r1;
      sred[warp][2] = r2;
    }
    __syncthreads();
    if (warp == 0) {
      const int nsc = (NX == 2) ? 3 : 1;
      for (int i = 0; i < nsc; ++i) {
        acc v;
        Ar::zero(v);
        if (lane < A_WARPS) v = sred[lane][i];
        v = warp_reduce<Ar>(v);
        if (lane == 0) pb[J * NX + i] = Ar::pack(v);
      }
    }
  }
  __threadfence();
  __syncthreads();
  if (tid == 0) s_last = (atomicAdd(&st->tickets[TK_DOT], 1u) == nblk - 1);
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  const int nout = J * NX + ((NX == 2) ? 3 : 1);
  const unsigned long long *pall = reinterpret_cast<const unsigned long long *>(a.part);
  for (int o = tid; o < nout; o += A_THREADS) {
    acc s;
    Ar::zero(s);
    for (int b = 0; b < nblk; ++b) Ar::merge(s, Ar::unpack(__ldcg(pall + (size_t)b * a.pstride + o)));
    res[o] = Ar::value(s);
  }
  __syncthreads();
  if (tid == 0) st->tickets[TK_DOT] = 0;
  gs_epilogue<NX>(a, res, mode);
}

template <int NX, int CPW, class Ar, class S>
__global__ void __launch_bounds__(A_THREADS, 1) k_gs_dot(StepArgs a, int mode) {
  gs_dot_body<NX, CPW, Ar, S>(a, mode, blockIdx.x, gridDim.x);
}

// Gram-Schmidt half A for bases wider than A_MAXJ columns: the columns in groups of A_WARPS * GW_CPW, each group a
// pass over the block's row tiles (u and w restaged per pass, one column's extra read per 128); per column the sum
// runs over the same rows in the same order as above.  The merged sums live in dynamic shared memory (2 J + 4
// doubles).
constexpr int GW_CPW = 8;
constexpr int GW_MAXJ = 1024;

template <int NX, class Ar, class S>
KS_DEVICE void gs_dot_wide_body(const StepArgs &a, int mode, int bid, int nblk) {
  KrylovState *st = a.st;
  if (st->stop) return;
  using val = typename Ar::val;
  using acc = typename Ar::acc;
  __shared__ __align__(16) val sx[NX][A_TILE];
  __shared__ acc sred[A_WARPS][3];
  __shared__ int s_last;
  extern __shared__ __align__(16) unsigned char gwraw[];
  double *res = reinterpret_cast<double *>(gwraw);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int n = a.n, J = a.J;
  const double sigma = st->sigma;
  using ST = typename S::T;
  const ST *Vb = static_cast<const ST *>(a.V);
  const ST *U = static_cast<const ST *>(a.U);
  const ST *W = static_cast<const ST *>(a.W);
  unsigned long long *pb = reinterpret_cast<unsigned long long *>(a.part) + (size_t)bid * a.pstride;
  acc sc0, sc1, sc2;
  Ar::zero(sc0);
  Ar::zero(sc1);
  Ar::zero(sc2);
  const int ntiles = (n + A_TILE - 1) / A_TILE;
  for (int g0 = 0; g0 < J; g0 += A_WARPS * GW_CPW) {
    acc cacc[GW_CPW][NX];
#pragma unroll
    for (int k = 0; k < GW_CPW; ++k)
#pragma unroll
      for (int q = 0; q < NX; ++q) Ar::zero(cacc[k][q]);
    for (int t = bid; t < ntiles; t += nblk) {
      const int r0 = t * A_TILE;
      const int rows = min(A_TILE, n - r0);
      {
        double u = 0.0, w = 0.0;
        if (tid < rows) {
          u = S::get(U + r0 + tid) * sigma;
          if (NX == 2) w = S::get(W + r0 + tid);
        }
        const val us = Ar::cvt(u);
        sx[0][tid] = us;
        if (g0 == 0) Ar::fma(sc0, us, us);
        if (NX == 2) {
          const val ws = Ar::cvt(w);
          sx[NX - 1][tid] = ws;
          if (g0 == 0) {
            Ar::fma(sc1, us, ws);
            Ar::fma(sc2, ws, ws);
          }
        }
      }
      __syncthreads();
#pragma unroll
      for (int k = 0; k < GW_CPW; ++k) {
        const int c = g0 + warp + k * A_WARPS;
        if (c < J) {
          const ST *col = Vb + (size_t)c * a.ldv + r0;
          if (rows == A_TILE) {
            val ca[8], cb[8];
#pragma unroll
            for (int i = 0; i < 8; ++i) S::template load2<Ar>(col + lane * 2 + 64 * i, ca[i], cb[i]);
#pragma unroll
            for (int i = 0; i < 8; ++i) {
              const int rr = lane * 2 + 64 * i;
              Ar::fma(cacc[k][0], ca[i], sx[0][rr]);
              Ar::fma(cacc[k][0], cb[i], sx[0][rr + 1]);
              if (NX == 2) {
                Ar::fma(cacc[k][NX - 1], ca[i], sx[NX - 1][rr]);
                Ar::fma(cacc[k][NX - 1], cb[i], sx[NX - 1][rr + 1]);
              }
            }
          } else {
            for (int rr = lane; rr < rows; rr += 32) {
              const val a0 = S::template load1<Ar>(col + rr);
              Ar::fma(cacc[k][0], a0, sx[0][rr]);
              if (NX == 2) Ar::fma(cacc[k][NX - 1], a0, sx[NX - 1][rr]);
            }
          }
        }
      }
      __syncthreads();
    }
#pragma unroll
    for (int k = 0; k < GW_CPW; ++k) {
      const int c = g0 + warp + k * A_WARPS;
      if (c < J) {
#pragma unroll
        for (int q = 0; q < NX; ++q) {
          const acc r = warp_reduce<Ar>(cacc[k][q]);
          if (lane == 0) pb[c * NX + q] = Ar::pack(r);
        }
      }
    }
  }
  {
    acc r0 = warp_reduce<Ar>(sc0), r1 = warp_reduce<Ar>(sc1), r2 = warp_reduce<Ar>(sc2);
    if (lane == 0) {
      sred[warp][0] = r0;
      sred[warp][1] = r1;
      sred[warp][2] = r2;
    }
    __syncthreads();
    if (warp == 0) {
      const int nsc = (NX == 2) ? 3 : 1;
      for (int i = 0; i < nsc; ++i) {
        acc v;
        Ar::zero(v);
        if (lane < A_WARPS) v = sred[lane][i];
        v = warp_reduce<Ar>(v);
        if (lane == 0) pb[J * NX + i] = Ar::pack(v);
      }
    }
  }
  __threadfence();
  __syncthreads();
  if (tid == 0) s_last = (atomicAdd(&st->tickets[TK_DOT], 1u) == nblk - 1);
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  const int nout = J * NX + ((NX == 2) ? 3 : 1);
  const unsigned long long *pall = reinterpret_cast<const unsigned long long *>(a.part);
  for (int o = tid; o < nout; o += A_THREADS) {
    acc s;
    Ar::zero(s);
    for (int b = 0; b < nblk; ++b) Ar::merge(s, Ar::unpack(__ldcg(pall + (size_t)b * a.pstride + o)));
    res[o] = Ar::value(s);
  }
  __syncthreads();
  if (tid == 0) st->tickets[TK_DOT] = 0;
  gs_epilogue<NX>(a, res, mode);
}

template <int NX, class Ar, class S>
__global__ void __launch_bounds__(A_THREADS, 1) k_gs_dot_wide(StepArgs a, int mode) {
  gs_dot_wide_body<NX, Ar, S>(a, mode, blockIdx.x, gridDim.x);
}

// ------------------------------------------------------------------------------------------------------------
// Gram-Schmidt half B: per row, v_j = (sigma u - V s) / nu and (NX = 2) w' = w - V g - tau sigma u, with ||w'||^2
// merged by the last block into the next step's scale.
// ------------------------------------------------------------------------------------------------------------
constexpr int B_THREADS = 256;
constexpr int B_TILE = 2 * B_THREADS;

template <int NX, class Ar, class S>
KS_DEVICE void gs_update_body(const StepArgs &a, int mode, int bid, int nblk) {
  KrylovState *st = a.st;
  if (st->stop) return;
  using val = typename Ar::val;
  using acc = typename Ar::acc;
  extern __shared__ __align__(16) unsigned char smraw[];
  val *cs = reinterpret_cast<val *>(smraw);  // s then g
  __shared__ acc sred[B_THREADS / 32];
  __shared__ int s_last;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int n = a.n, J = a.J;
  for (int i = tid; i < NX * J; i += B_THREADS) cs[i] = Ar::cvt(a.coef[i]);
  __syncthreads();
  const double sigma = st->sigma, invnu = st->invnu, tsig = st->tau_sigma;
  using ST = typename S::T;
  const ST *Vb = static_cast<const ST *>(a.V);
  ST *U = static_cast<ST *>(a.U);
  ST *W = static_cast<ST *>(a.W);
  acc nrm;
  Ar::zero(nrm);
  const int ntiles = (n + B_TILE - 1) / B_TILE;
  for (int t = bid; t < ntiles; t += nblk) {
    const int r = t * B_TILE + tid * 2;
    if (r + 1 < n) {
      acc s0, s1, g0, g1;
      Ar::zero(s0);
      Ar::zero(s1);
      Ar::zero(g0);
      Ar::zero(g1);
      const ST *col = Vb + r;
      // groups of 8 columns, the next group's loads in flight while the current one is consumed
      val xa[8], xb[8];
#pragma unroll
      for (int q = 0; q < 8; ++q)
        if (q < J) S::template load2<Ar>(col + (size_t)q * a.ldv, xa[q], xb[q]);
      for (int c0 = 0; c0 < J; c0 += 8) {
        val ca[8], cb[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          ca[q] = xa[q];
          cb[q] = xb[q];
        }
#pragma unroll
        for (int q = 0; q < 8; ++q)
          if (c0 + 8 + q < J) S::template load2<Ar>(col + (size_t)(c0 + 8 + q) * a.ldv, xa[q], xb[q]);
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          if (c0 + q < J) {
            Ar::fma(s0, ca[q], cs[c0 + q]);
            Ar::fma(s1, cb[q], cs[c0 + q]);
            if (NX == 2) {
              Ar::fma(g0, ca[q], cs[J + c0 + q]);
              Ar::fma(g1, cb[q], cs[J + c0 + q]);
            }
          }
        }
      }
      double ux, uy;
      S::get2(U + r, ux, uy);
      S::put2(U + r, (sigma * ux - Ar::value(s0)) * invnu, (sigma * uy - Ar::value(s1)) * invnu);
      if (NX == 2) {
        double wx, wy;
        S::get2(W + r, wx, wy);
        const double ox = wx - Ar::value(g0) - tsig * ux, oy = wy - Ar::value(g1) - tsig * uy;
        S::put2(W + r, ox, oy);
        const val w0 = Ar::cvt(ox), w1 = Ar::cvt(oy);
        Ar::fma(nrm, w0, w0);
        Ar::fma(nrm, w1, w1);
      }
    } else if (r < n) {
      acc s0, g0;
      Ar::zero(s0);
      Ar::zero(g0);
      for (int c = 0; c < J; ++c) {
        const val v0 = S::template load1<Ar>(Vb + r + (size_t)c * a.ldv);
        Ar::fma(s0, v0, cs[c]);
        if (NX == 2) Ar::fma(g0, v0, cs[J + c]);
      }
      const double u = S::get(U + r);
      S::put(U + r, (sigma * u - Ar::value(s0)) * invnu);
      if (NX == 2) {
        const double wo = S::get(W + r) - Ar::value(g0) - tsig * u;
        S::put(W + r, wo);
        const val w0 = Ar::cvt(wo);
        Ar::fma(nrm, w0, w0);
      }
    }
  }
  if (NX == 1) return;  // no norm needed after the final reorthogonalisation or a start-vector pass
  nrm = warp_reduce<Ar>(nrm);
  if (lane == 0) sred[warp] = nrm;
  __syncthreads();
  unsigned long long *pb = reinterpret_cast<unsigned long long *>(a.part);
  if (warp == 0) {
    acc v;
    Ar::zero(v);
    if (lane < B_THREADS / 32) v = sred[lane];
    v = warp_reduce<Ar>(v);
    if (lane == 0) pb[bid] = Ar::pack(v);
  }
  __threadfence();
  __syncthreads();
  if (tid == 0) s_last = (atomicAdd(&st->tickets[TK_UPD], 1u) == nblk - 1);
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  if (warp == 0) {
    acc v;
    Ar::zero(v);
    for (int b = lane; b < nblk; b += 32) Ar::merge(v, Ar::unpack(__ldcg(pb + b)));
    // merge lanes in a fixed order
    v = warp_reduce<Ar>(v);
    if (lane == 0) {
      const double beta = sqrt(Ar::value(v));
      st->tickets[TK_UPD] = 0;
      if (beta == 0.0 || !(beta == beta)) {
        st->stop = 1;
        st->breakdown = 1;
        st->m = a.j + 1;
        st->beta_out = 0.0;
        if (a.hermitian) a.e[a.j] = 0.0;
        else a.H[(a.j + 1) + (size_t)a.j * a.ldh] = 0.0;
      } else {
        st->sigma = 1.0 / beta;
        st->beta_prev = beta * st->invnu;
      }
    }
  }
}

template <int NX, class Ar, class S>
__global__ void __launch_bounds__(B_THREADS) k_gs_update(StepArgs a, int mode) {
  gs_update_body<NX, Ar, S>(a, mode, blockIdx.x, gridDim.x);
}

// ------------------------------------------------------------------------------------------------------------
// Thick restart: V(:, s0:s0+N) = V(:, a0:a0+K) * Q(a0:a0+K, s0:s0+N), in place by row tiles.
// ------------------------------------------------------------------------------------------------------------
constexpr int R_THREADS = 256;
constexpr int R_ROWS = 32;
constexpr int R_MAXN = 144;

// Thread (ty, tx) of a restart block owns rows 2ty + 32p and 2ty + 1 + 32p of a tile (p < RP) and columns
// tx + 16q (q < CQ): CQ = ceil(N / 16) column chunks, and RP row pairs per thread, more when N is small, so a tile
// holds 32 RP rows.  Every output element is one thread's sum over k in increasing order, whatever the tiling.
template <int CQ>
__host__ __device__ constexpr int restart_rp() { return CQ <= 2 ? 4 : (CQ <= 4 ? 2 : 1); }
template <int CQ>
__host__ __device__ constexpr int restart_tile_rows() { return 32 * restart_rp<CQ>(); }

template <class Ar, class S, int CQ>
KS_DEVICE void restart_body(typename S::T *V, long long ldv, int n, int a0, int K, int s0, int N, const double *Q,
                            int ldq, int bid, int nblk) {
  using val = typename Ar::val;
  using acc = typename Ar::acc;
  constexpr int RP = restart_rp<CQ>(), TR = restart_tile_rows<CQ>();
  extern __shared__ __align__(16) unsigned char smraw[];
  val *Qs = reinterpret_cast<val *>(smraw);  // K x N, row k contiguous
  val *Vt = Qs + (size_t)K * N;              // K x TR, column k contiguous
  const int tid = threadIdx.x;
  for (int i = tid; i < K * N; i += R_THREADS) {
    const int k = i / N, c = i % N;
    Qs[i] = Ar::cvt(Q[(a0 + k) + (size_t)(s0 + c) * ldq]);
  }
  const int ty = tid / 16, tx = tid % 16;
  const int ntiles = (n + TR - 1) / TR;
  for (int t = bid; t < ntiles; t += nblk) {
    const int r0 = t * TR;
    const int rows = min(TR, n - r0);
    __syncthreads();
    for (int i = tid; i < K * TR; i += R_THREADS) {
      const int k = i / TR, r = i % TR;
      Vt[i] = (r < rows) ? S::template load1<Ar>(V + (r0 + r) + (size_t)(a0 + k) * ldv) : Ar::cvt(0.0);
    }
    __syncthreads();
    acc o0[CQ][RP], o1[CQ][RP];
#pragma unroll
    for (int q = 0; q < CQ; ++q)
#pragma unroll
      for (int p = 0; p < RP; ++p) {
        Ar::zero(o0[q][p]);
        Ar::zero(o1[q][p]);
      }
    for (int k = 0; k < K; ++k) {
      val v0[RP], v1[RP];
#pragma unroll
      for (int p = 0; p < RP; ++p) {
        v0[p] = Vt[k * TR + 2 * ty + 32 * p];
        v1[p] = Vt[k * TR + 2 * ty + 1 + 32 * p];
      }
#pragma unroll
      for (int q = 0; q < CQ; ++q) {
        const int c = tx + 16 * q;
        if (c < N) {
          const val qq = Qs[k * N + c];
#pragma unroll
          for (int p = 0; p < RP; ++p) {
            Ar::fma(o0[q][p], v0[p], qq);
            Ar::fma(o1[q][p], v1[p], qq);
          }
        }
      }
    }
    __syncthreads();  // every read of this tile's V columns precedes the in-place writes
#pragma unroll
    for (int q = 0; q < CQ; ++q) {
      const int c = tx + 16 * q;
      if (c < N) {
#pragma unroll
        for (int p = 0; p < RP; ++p) {
          const int r = 2 * ty + 32 * p;
          if (r < rows) S::put(V + (r0 + r) + (size_t)(s0 + c) * ldv, Ar::value(o0[q][p]));
          if (r + 1 < rows) S::put(V + (r0 + r + 1) + (size_t)(s0 + c) * ldv, Ar::value(o1[q][p]));
        }
      }
    }
  }
}

// The restart for K or N above R_MAXN: tiles of RW_ROWS rows, the tile's K values per row staged in shared memory
// (K x RW_ROWS, up to 128 KB), Q read through the cache.  Thread (cl, r) owns row r of the tile and output columns
// cl + 16 q, in chunks of RW_CQ; every output element is one thread's sum over k in increasing order.  All reads of
// the tile's rows precede the block's in-place writes (the tile is in shared memory), and no two blocks share a row.
constexpr int RW_ROWS = 16;
constexpr int RW_CQ = 8;
constexpr int RW_MAXK = 1024;

template <class Ar, class S>
KS_DEVICE void restart_wide_body(typename S::T *V, long long ldv, int n, int a0, int K, int s0, int N,
                                 const double *__restrict__ Q, int ldq, int bid, int nblk) {
  using val = typename Ar::val;
  using acc = typename Ar::acc;
  extern __shared__ __align__(16) unsigned char smraw[];
  val *Vt = reinterpret_cast<val *>(smraw);  // K x RW_ROWS, column k contiguous
  const int tid = threadIdx.x;
  const int r = tid % RW_ROWS, cl = tid / RW_ROWS;
  constexpr int NCL = R_THREADS / RW_ROWS;
  const int ntiles = (n + RW_ROWS - 1) / RW_ROWS;
  for (int t = bid; t < ntiles; t += nblk) {
    const int r0 = t * RW_ROWS;
    const int rows = min(RW_ROWS, n - r0);
    __syncthreads();
    for (int i = tid; i < K * RW_ROWS; i += R_THREADS) {
      const int k = i / RW_ROWS, rr = i % RW_ROWS;
      Vt[i] = (rr < rows) ? S::template load1<Ar>(V + (r0 + rr) + (size_t)(a0 + k) * ldv) : Ar::cvt(0.0);
    }
    __syncthreads();
    for (int cb = 0; cb < N; cb += NCL * RW_CQ) {
      acc o[RW_CQ];
#pragma unroll
      for (int q = 0; q < RW_CQ; ++q) Ar::zero(o[q]);
      for (int k = 0; k < K; ++k) {
        const val v = Vt[k * RW_ROWS + r];
        const double *qk = Q + (a0 + k) + (size_t)s0 * ldq;
#pragma unroll
        for (int q = 0; q < RW_CQ; ++q) {
          const int c = cb + cl + NCL * q;
          if (c < N) Ar::fma(o[q], v, Ar::cvt(__ldg(qk + (size_t)c * ldq)));
        }
      }
      if (r < rows) {
#pragma unroll
        for (int q = 0; q < RW_CQ; ++q) {
          const int c = cb + cl + NCL * q;
          if (c < N) S::put(V + (r0 + r) + (size_t)(s0 + c) * ldv, Ar::value(o[q]));
        }
      }
    }
  }
}

template <class Ar, class S>
__global__ void __launch_bounds__(R_THREADS, 1) k_restart_wide(typename S::T *V, long long ldv, int n, int a0, int K,
                                                               int s0, int N, const double *Q, int ldq) {
  restart_wide_body<Ar, S>(V, ldv, n, a0, K, s0, N, Q, ldq, blockIdx.x, gridDim.x);
}

template <class Ar, class S, int CQ>
__global__ void __launch_bounds__(R_THREADS, 2) k_restart(typename S::T *V, long long ldv, int n, int a0, int K,
                                                          int s0, int N, const double *Q, int ldq) {
  restart_body<Ar, S, CQ>(V, ldv, n, a0, K, s0, N, Q, ldq, blockIdx.x, gridDim.x);
}

}  // namespace ksg
