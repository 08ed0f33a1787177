// common.cuh -- shared device helpers for the GB300 Krylov-Schur kernels.
//
// FP64-accurate arithmetic on the FP32 pipes.  GB300's FP64 pipe delivers ~1.2 TFLOP/s (measured: DFMA and
// DMMA alike) against ~75 TFLOP/s FP32, so a streaming pass that spends one DFMA per 8-byte element tops out
// at ~3.9 TB/s, below the ~6.8 TB/s HBM rate.  The bandwidth-bound kernels therefore keep FP64 storage but do
// their products and sums on FP32 pairs with error-free transformations:
//   * split:      a double v becomes hi + lo (two floats, 47 significant bits) using integer operations only
//                 (F2F conversions run on the FP64 pipe on this part);
//   * TwoProduct: a*b = p + e exactly with p = fl(a*b), e = fma(a, b, -p)            (Dekker 1971, via FMA);
//   * TwoSum:     a+b = s + t exactly                                                  (Knuth, TAOCP vol. 2).
// A product of two split values keeps a relative error below 2^-46; sums carry a (hi, lo) accumulator.
// Coefficient algebra, norms' square roots and the projected problem stay in true FP64.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#define KS_DEVICE __device__ __forceinline__

struct f2x {
  float hi, lo;
};

// Split a double into hi + lo floats with integer operations.  hi keeps the top 24 significand bits
// (truncated), lo the next 23 (truncated).  |v| < 2^-126 flushes to zero (and lo flushes below 2^-103): such
// entries contribute below 2^-100 of a unit vector's norm.  |v| >= 2^128 is outside the supported range; the
// solver scales the operator by a power of two so that vectors stay well inside it.
KS_DEVICE f2x split_f64(double v) {
  unsigned long long b = (unsigned long long)__double_as_longlong(v);
  unsigned H = (unsigned)(b >> 32), L = (unsigned)b;
  unsigned sign = H & 0x80000000u;
  unsigned Ha = (H & 0x7fffffffu) - (896u << 20);  // exponent rebased to binary32 (valid for 1..254)
  unsigned hib = __funnelshift_l(L, Ha, 3) | sign;   // (Ha << 3) | (L >> 29)
  unsigned ebias = (Ha - (23u << 20)) & 0x7ff00000u;  // (e_32 - 23) << 20 (masked garbage when e_32 <= 23)
  unsigned elo = ebias << 3;
  float F = __uint_as_float(elo | ((L >> 6) & 0x7fffffu));
  float lo = F - __uint_as_float(elo);
  int e32 = (int)(Ha >> 20);  // negative values wrap to large unsigned; cast and test below
  f2x r;
  r.hi = ((int)Ha > 0 && e32 >= 1) ? __uint_as_float(hib) : 0.0f;
  float los = __uint_as_float(__float_as_uint(lo) ^ sign);
  r.lo = ((int)Ha >= (int)(24u << 20)) ? los : 0.0f;
  return r;
}

KS_DEVICE f2x split_f32(float v) {
  f2x r;
  r.hi = v;
  r.lo = 0.0f;
  return r;
}

// Accumulator for sum_i a_i*b_i with a, b split values.
struct dfacc {
  float s, c;  // s: running high sum, c: compensation (all rounding errors and the low-order products)
};

KS_DEVICE void acc_zero(dfacc &a) {
  a.s = 0.0f;
  a.c = 0.0f;
}

// a += x*y (x, y split).  TwoProduct on the high parts, the cross terms in FP32, TwoSum into the accumulator.
KS_DEVICE void acc_fma(dfacc &a, f2x x, f2x y) {
  float p = x.hi * y.hi;
  float e = __fmaf_rn(x.hi, y.hi, -p);
  e = __fmaf_rn(x.hi, y.lo, __fmaf_rn(x.lo, y.hi, e));
  float s = a.s + p;
  float bp = s - a.s;
  float err = (a.s - (s - bp)) + (p - bp);
  a.s = s;
  a.c += err + e;
}

// a += x (x split)
KS_DEVICE void acc_add(dfacc &a, f2x x) {
  float s = a.s + x.hi;
  float bp = s - a.s;
  float err = (a.s - (s - bp)) + (x.hi - bp);
  a.s = s;
  a.c += err + x.lo;
}

// a += b (accumulators)
KS_DEVICE void acc_merge(dfacc &a, dfacc b) {
  float s = a.s + b.s;
  float bp = s - a.s;
  float err = (a.s - (s - bp)) + (b.s - bp);
  a.s = s;
  a.c += err + b.c;
}

KS_DEVICE double acc_value(dfacc a) { return (double)a.s + (double)a.c; }

KS_DEVICE dfacc shfl_down_acc(dfacc a, int off) {
  dfacc r;
  r.s = __shfl_down_sync(0xffffffffu, a.s, off);
  r.c = __shfl_down_sync(0xffffffffu, a.c, off);
  return r;
}

KS_DEVICE dfacc warp_reduce_acc(dfacc a) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) acc_merge(a, shfl_down_acc(a, off));
  return a;
}

// Streaming loads that do not displace the L2-resident vectors (x of the SpMV, u and w).
KS_DEVICE double2 ld_stream2(const double *p) { return __ldcs(reinterpret_cast<const double2 *>(p)); }
KS_DEVICE double ld_stream(const double *p) { return __ldcs(p); }
