// gs_fixed.cuh -- fixed-point helpers of the Gram-Schmidt pairs for IEEE-double storage that compute every product
// exactly (k_gs_tc.cu on the tensor cores, k_gs_ix.cu on the integer pipes): scale exponents, the exponent table of
// the basis columns, 128-bit integer sums and their conversion back to doubles, double-double sums.
#pragma once

#include <limits.h>

#include "common.cuh"
#include "kernels.h"
#include "tc_common.cuh"

namespace ksg {

// scale exponent of a value: |v| < 2^(E - 1022) for its biased exponent E >= 1; recorded in [-127, 127], -128 for zero
KS_DEVICE int gt_expo(double v) { return (int)(((unsigned long long)__double_as_longlong(v) >> 52) & 0x7FF); }
KS_DEVICE int gt_escale(int Emax) {
  if (Emax == 0) return -128;
  const int e = Emax - 1022;
  return e < -127 ? -127 : (e > 127 ? 127 : e);
}

// 2^k as a double over the whole exponent range used here (|k| < 1100)
KS_DEVICE double gt_pow2(int k) { return t5_pow2(k); }

// 128-bit two's complement (hi, lo) helpers
KS_DEVICE void gt_add128(long long &hi, unsigned long long &lo, long long bhi, unsigned long long blo) {
  const unsigned long long s = lo + blo;
  hi = hi + bhi + (s < lo ? 1 : 0);
  lo = s;
}
// the value of a 128-bit integer as a double (two roundings at most: within 1 ulp)
KS_DEVICE double gt_to_double(long long hi, unsigned long long lo) {
  return fma(__ll2double_rn(hi), 18446744073709551616.0, __ull2double_rn(lo));
}

// double-double accumulation (TwoSum)
KS_DEVICE void gt_dd_add(double &hi, double &lo, double x) {
  const double s = hi + x;
  const double bb = s - hi;
  lo += (hi - (s - bb)) + (x - bb);
  hi = s;
}

// the recorded scale of V column j over tiles [t0, t0 + nt): the largest exponent (-128 when every tile is zero)
KS_DEVICE int gt_vscale(const GTArgs &g, int j, int t0, int nt) {
  int e = -128;
  const signed char *p = g.vexp + (size_t)j * g.ldt + t0;
  for (int t = 0; t < nt; ++t) e = max(e, (int)p[t]);
  return e;
}

// ---------------------------------------------------------------------------------------------------------------
// The integer-pipe form (k_gs_ix.cu)
// ---------------------------------------------------------------------------------------------------------------

// X = trunc(v 2^(53 - e)), |X| < 2^53 when |v| < 2^e (the full significand of every value in the top binade
// [2^(e-1), 2^e), fewer bits below), returned as X = H 2^26 + L with the sign of v on both halves (|H| < 2^27,
// |L| < 2^26).  Integer operations only.  A value at or above 2^e (or not finite) makes *flag negative.
KS_DEVICE void ix_split53(double v, int e, int &H, int &L, int &flag) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(v);
  const unsigned hw = (unsigned)(u >> 32);
  const int E = (int)((hw >> 20) & 0x7FFu);
  const int s0 = 1022 + e - E;  // |X| = m >> s0 for m = 2^52 | fraction (zero and subnormals shift out entirely)
  flag |= s0;
  const unsigned long long m =
      ((unsigned long long)((hw & 0xFFFFFu) | 0x100000u) << 32) | (unsigned long long)(unsigned)u;
  const unsigned long long x = m >> min((unsigned)s0, 63u);
  const int sm = (int)hw >> 31;  // 0, or -1 for a negative value
  H = ((int)(x >> 26) ^ sm) - sm;
  L = ((int)((unsigned)x & 0x3FFFFFFu) ^ sm) - sm;
}

// The exact sum P = hh 2^52 + mm 2^26 + ll of a run of split products, as a 128-bit integer.
KS_DEVICE void ix_combine(long long hh, long long mm, long long ll, long long &hi, unsigned long long &lo) {
  hi = hh >> 12;
  lo = (unsigned long long)hh << 52;
  gt_add128(hi, lo, mm >> 38, (unsigned long long)mm << 26);
  gt_add128(hi, lo, ll >> 63, (unsigned long long)ll);
}

// arithmetic right shift of a 128-bit integer by 0 <= s <= 127
KS_DEVICE void ix_sra128(long long &hi, unsigned long long &lo, int s) {
  if (s >= 64) {
    lo = (unsigned long long)(hi >> (s - 64));
    hi >>= 63;
  } else if (s > 0) {
    lo = (lo >> s) | ((unsigned long long)hi << (64 - s));
    hi >>= s;
  }
}

// A 128-bit accumulator with a binary exponent: the value is (hi, lo) 2^k (k == INT_MIN: empty).  ix_acc_add adds
// P 2^kp: the operand with the smaller exponent is shifted right to the larger (the bits dropped lie below 2^-106
// of the larger operand's scale), and the accumulator keeps |(hi, lo)| < 2^124.
struct IxAcc {
  long long hi;
  unsigned long long lo;
  int k;
};
KS_DEVICE void ix_acc_zero(IxAcc &A) {
  A.hi = 0;
  A.lo = 0;
  A.k = INT_MIN;
}
KS_DEVICE void ix_acc_add(IxAcc &A, long long phi, unsigned long long plo, int kp) {
  if (phi == 0 && plo == 0) return;
  if (A.k == INT_MIN) {
    A.hi = phi;
    A.lo = plo;
    A.k = kp;
  } else {
    if (kp > A.k) {
      ix_sra128(A.hi, A.lo, min(kp - A.k, 127));
      A.k = kp;
    } else if (kp < A.k) {
      ix_sra128(phi, plo, min(A.k - kp, 127));
    }
    gt_add128(A.hi, A.lo, phi, plo);
  }
  if ((A.hi >> 59) != (A.hi >> 63)) {
    ix_sra128(A.hi, A.lo, 4);
    A.k += 4;
  }
}

// (hi, lo) 2^k rounded once to the nearest double (ties to even), by integer operations; results outside the
// normal range go through ldexp
KS_DEVICE double ix_to_double(long long hi, unsigned long long lo, int k) {
  const bool neg = hi < 0;
  unsigned long long h = (unsigned long long)hi;
  if (neg) {
    lo = ~lo + 1ull;
    h = ~h + (lo == 0ull ? 1ull : 0ull);
  }
  if (h == 0ull && lo == 0ull) return 0.0;
  int sh = 0;
  if (h == 0ull) {
    h = lo;
    lo = 0ull;
    sh = 64;
  }
  const int lz = __clzll((long long)h);
  if (lz > 0) {
    h = (h << lz) | (lo >> (64 - lz));
    lo <<= lz;
  }
  sh += lz;
  // value = (h, lo) 2^(k - sh) with bit 63 of h set: the top 53 bits, then round to nearest even
  unsigned long long m = h >> 11;
  const unsigned long long rest = h & 0x7FFull;
  if ((rest & 0x400ull) && ((rest & 0x3FFull) || lo || (m & 1ull))) ++m;
  int e2 = k - sh + 75;  // value = m 2^e2
  if (m >> 53) {
    m >>= 1;
    ++e2;
  }
  const int be = e2 + 1075;
  if (be < 1 || be > 2046) return ldexp(neg ? -(double)m : (double)m, e2);
  return __longlong_as_double((long long)(((unsigned long long)neg << 63) | ((unsigned long long)be << 52) |
                                          (m & 0xFFFFFFFFFFFFFull)));
}

}  // namespace ksg
