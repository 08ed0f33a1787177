// oz_round.h -- integer-only pieces of the FP64 epilogue of the tcgen05 restart, usable on the host (for the CPU
// tests that pin them) and the device.
//
// The restart's level sums come out of the tensor cores as FP32 values that are exact integers below 2^24 in
// magnitude; the FP64-storage epilogue combines them into X = H 2^42 + R (|H| < 2^33, |R| < 2^61) and writes
// X 2^sc rounded to a double.  On GB300 a warp-wide FP64 instruction occupies the FP64 pipe of its sub-partition for
// about 64 cycles, so both steps run on the integer units instead:
//   oz_f2i_exact   the integer value of an integer-valued float (exponent and significand fields)
//   oz_round_x     X 2^sc correctly rounded (to nearest, ties to even) from the 128-bit two's complement of X:
//                  the top 53 bits of |X|, the rounding decision from the bits below, the exponent assembled.
//                  Returns false when the result would leave the normal range (the caller computes it in FP64).
#pragma once

#include <stdint.h>

#ifdef __CUDACC__
#define OZ_HD __host__ __device__ __forceinline__
#else
#define OZ_HD inline
#endif

OZ_HD int oz_clz64(uint64_t x) {
#ifdef __CUDA_ARCH__
  return __clzll((long long)x);
#else
  return x ? __builtin_clzll(x) : 64;
#endif
}

OZ_HD uint32_t oz_float_bits(float f) {
#ifdef __CUDA_ARCH__
  return __float_as_uint(f);
#else
  uint32_t u;
  __builtin_memcpy(&u, &f, 4);
  return u;
#endif
}

OZ_HD double oz_double_from_bits(uint64_t b) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)b);
#else
  double d;
  __builtin_memcpy(&d, &b, 8);
  return d;
#endif
}

// an integer-valued float with |f| < 2^24 as an integer
OZ_HD int32_t oz_f2i_exact(float f) {
  const uint32_t u = oz_float_bits(f);
  const int e = (int)((u >> 23) & 0xFFu);
  if (e < 127) return 0;  // +-0 (the only integer below 1 in magnitude)
  const int32_t m = (int32_t)((u & 0x7FFFFFu) | 0x800000u) >> (150 - e);
  return (u >> 31) ? -m : m;
}

// X 2^sc with X = H 2^42 + R, correctly rounded to a double; false when the result is not a normal double
OZ_HD bool oz_round_x(int64_t H, int64_t R, int sc, double *out) {
  // X as 128-bit two's complement (hi, lo)
  const uint64_t lh = (uint64_t)H << 42;
  const uint64_t hh = (uint64_t)(H >> 22);  // arithmetic shift: the sign extends
  const uint64_t lr = (uint64_t)R;
  const uint64_t hr = (uint64_t)(R >> 63);
  uint64_t lo = lh + lr;
  uint64_t hi = hh + hr + (lo < lh ? 1u : 0u);
  const uint64_t neg = hi >> 63;
  if (neg) {
    lo = ~lo + 1u;
    hi = ~hi + (lo == 0 ? 1u : 0u);
  }
  if ((hi | lo) == 0) {
    *out = 0.0;
    return true;
  }
  // position of the leading bit; |X| < 2^76, so p <= 75 and the shift below stays under 64
  const int p = hi ? 127 - oz_clz64(hi) : 63 - oz_clz64(lo);
  uint64_t mant;
  int e = p;
  if (p <= 52) {
    mant = lo << (52 - p);
  } else {
    const int sh = p - 52;  // 1 .. 23
    mant = (lo >> sh) | (hi << (64 - sh));
    const uint64_t rem = lo & ((1ull << sh) - 1u);
    const uint64_t half = 1ull << (sh - 1);
    if (rem > half || (rem == half && (mant & 1u))) {
      mant += 1u;
      if (mant >> 53) {
        mant >>= 1;
        e += 1;
      }
    }
  }
  const int biased = e + sc + 1023;
  if (biased < 1 || biased > 2046) return false;
  *out = oz_double_from_bits((neg << 63) | ((uint64_t)biased << 52) | (mant & 0xFFFFFFFFFFFFFull));
  return true;
}
