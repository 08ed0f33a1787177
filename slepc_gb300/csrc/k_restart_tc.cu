// k_restart_tc.cu -- the thick restart V(:, s0:s0+N) = V(:, a0:a0+K) Q on the bf16 tensor cores, to FP64-class
// accuracy, by an error-free split of both factors (the scheme of Ozaki, Ogita, Oishi and Rump, "Error-free
// transformations of matrix multiplication by using fast routines of matrix multiplication and its applications",
// Numer. Algorithms 59, 2012):
//
//   row r of the V tile:   v / 2^e_r = sum_{s<8} a_s 2^(-7(s+1)),   a_s integers in [-127, 127]
//   column c of Q:         q / 2^f_c = sum_{t<7} b_t 2^(-7(t+1)),   b_t integers in [-128, 128]
//   v q = 2^(e_r + f_c) sum_L 2^(-7(L+2)) P_L,   P_L = sum_{s+t=L} sum_k a_s b_t   (L <= 7; dropped terms < 2^-63)
//
// V keeps 56 bits below its row maximum (rows of a Krylov basis can span many orders of magnitude), Q 49 bits below
// its column maximum.  Every a_s and b_t is exact in bf16, every product exact, and a level has at most 7 terms, so
// |P_L| <= 7 * 127 * 128 * 144 < 2^24 and the FP32 accumulation of the tensor cores is exact (measured on GB300,
// sums up to 1.63e7).  The 35 slice products run as mma.sync m16n8k16 (609 TFLOP/s measured); the eight level sums
// are recombined exactly in FP32 pairs and scaled back.
// The 49-bit fixed point of a pair value is formed with integer operations on its float bits, so nothing touches the
// FP64 pipe in the main kernel.
#include <cuda_bf16.h>

#include <type_traits>

#include "common.cuh"
#include "kernels.h"
#include "ks_types.h"
#include "tc_common.cuh"

namespace ksg {

constexpr int OZ_SA = 8;         // slices of V (56 bits)
constexpr int OZ_S = 7;          // slices of Q (49 bits) for pair storage and for FP64 storage with K > 128
constexpr int OZ_QMAX = 8;       // slices of Q (56 bits) for FP64 storage with K <= 128; the scratch holds 8
constexpr int OZ_L = 8;          // levels s + t kept
constexpr int OZ_ROWS = 64;      // rows of V per tile
constexpr int OZ_THREADS = 256;  // 8 warps: 4 row groups of 16 x 2 column halves of a chunk
constexpr int OZ_NC = 32;        // output columns per chunk (4 mma n-tiles)
constexpr int OZ_PAD = 8;        // bf16 padding per row of the Q slices (rows stay 16-byte aligned for 16-byte copies)
constexpr int OZ_PADA = 2;       // bf16 padding per row of the V slices: an odd word stride, so the slicing pass's
                                 // stores from 32 consecutive rows hit 32 banks

size_t restart_tc_scratch_bytes(int ld) {
  const int kp = (ld + 15) / 16 * 16, np = (ld + OZ_NC - 1) / OZ_NC * OZ_NC;
  return (size_t)OZ_QMAX * np * kp * sizeof(__nv_bfloat16) + (size_t)np * sizeof(int) + 256;
}

static size_t oz_smem_bytes(int kp) {
  return ((size_t)OZ_SA * OZ_ROWS * (kp + OZ_PADA) + (size_t)OZ_S * OZ_NC * (kp + OZ_PAD)) *
             sizeof(__nv_bfloat16) +
         OZ_ROWS * sizeof(int) + 16;
}

// Column exponents and qs slices of Q(a0 + k, s0 + c), k < K, c < N (zero-padded to kp x np): one block per column.
// q / 2^f is rounded to a 7 qs-bit fixed point and cut into 7-bit slices, most significant first.
// Layout of slice t: [c][k] (cm = 0, the mma.sync kernel), or K-major core matrices [k/8][c/8][c%8][k%8] (cm = 1, the
// tcgen05 kernel: the 8-column groups of one k-group are contiguous, so a stage is a few bulk copies).
__global__ void k_oz_qslice(const double *__restrict__ Q, int ldq, int a0, int s0, int K, int N, int kp, int np,
                            __nv_bfloat16 *__restrict__ B, int *__restrict__ fcol, int cmlayout, int qs) {
  __shared__ double red[32];
  const int c = blockIdx.x;
  const bool col_ok = c < N;
  double mx = 0.0;
  if (col_ok)
    for (int k = threadIdx.x; k < K; k += blockDim.x) mx = fmax(mx, fabs(Q[(a0 + k) + (size_t)(s0 + c) * ldq]));
  for (int off = 16; off > 0; off >>= 1) mx = fmax(mx, __shfl_down_sync(0xffffffffu, mx, off));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mx;
  __syncthreads();
  if (threadIdx.x == 0) {
    double m = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) m = fmax(m, red[w]);
    red[0] = m;
  }
  __syncthreads();
  const double cm = red[0];
  const int f = (cm > 0.0) ? ilogb(cm) + 1 : 0;  // |q| / 2^f < 1
  if (threadIdx.x == 0) fcol[c] = f;
  const int bits = 7 * qs;
  for (int k = threadIdx.x; k < kp; k += blockDim.x) {
    long long y = 0;
    if (col_ok && k < K) y = __double2ll_rn(scalbn(Q[(a0 + k) + (size_t)(s0 + c) * ldq], bits - f));
    const bool neg = y < 0;
    const unsigned long long a = neg ? (unsigned long long)(-y) : (unsigned long long)y;
    for (int t = 0; t < qs; ++t) {
      // 7-bit slices; only the top one may reach 128 (when |q| 2^(bits-f) rounds up to 2^bits)
      const int sl = (int)((a >> (bits - 7 - 7 * t)) & (t == 0 ? 255ull : 127ull));
      const size_t at = cmlayout ? (((size_t)t * (kp / 8) + k / 8) * (np / 8) + c / 8) * 64 + (c % 8) * 8 + (k % 8)
                           : ((size_t)t * np + c) * kp + k;
      B[at] = __float2bfloat16_rn(neg ? -(float)sl : (float)sl);
    }
  }
}

// signed 56-bit fixed point of x * 2^(56 - e), |x| < 2^e, from the float's bits (truncated below 2^-56)
KS_DEVICE long long oz_fix56(float x, int e) {
  const unsigned u = __float_as_uint(x);
  const int E = (int)((u >> 23) & 0xFFu);
  if (E == 0) return 0;
  const long long m = (long long)((u & 0x7FFFFFu) | 0x800000u);
  const int sh = (E - 150) + 56 - e;
  long long r;
  if (sh >= 0) r = sh < 40 ? (m << sh) : 0;
  else r = sh > -40 ? (m >> (-sh)) : 0;
  return (u >> 31) ? -r : r;
}

KS_DEVICE void oz_mma(float *d, const unsigned *a, const unsigned *b) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// (s, c) += x exactly as a pair (TwoSum)
KS_DEVICE void oz_add(float &s, float &c, float x) {
  const float t = s + x;
  const float z = t - s;
  c += (s - (t - z)) + (x - z);
  s = t;
}

__global__ void __launch_bounds__(OZ_THREADS, 1) k_restart_tc(float2 *__restrict__ V, long long ldv, int n, int a0,
                                                               int K, int s0, int N, int kp, int np,
                                                               const __nv_bfloat16 *__restrict__ Bsl,
                                                               const int *__restrict__ fcol) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const int lda = kp + OZ_PADA, ldb = kp + OZ_PAD;
  __nv_bfloat16 *As = reinterpret_cast<__nv_bfloat16 *>(smraw);  // [s][r][k]
  // Q slices after the V slices, rounded up to a 16-byte boundary
  const size_t aoff = ((size_t)OZ_SA * OZ_ROWS * lda * sizeof(__nv_bfloat16) + 15) / 16 * 16;
  __nv_bfloat16 *Bs = reinterpret_cast<__nv_bfloat16 *>(smraw + aoff);  // [t][c][k]
  int *erow = reinterpret_cast<int *>(Bs + (size_t)OZ_S * OZ_NC * ldb);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int g = lane >> 2, tq = lane & 3;
  const int rg = warp >> 1, half = warp & 1;
  const int ntiles = (n + OZ_ROWS - 1) / OZ_ROWS;
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int r0 = tile * OZ_ROWS;
    const int rows = min(OZ_ROWS, n - r0);
    __syncthreads();  // the previous tile's smem is free
    if (tid < OZ_ROWS) erow[tid] = 0;
    __syncthreads();
    // 1. row exponents: e_r = 1 + floor(log2 max_k |hi|), from the float exponent fields
    for (int i = tid; i < OZ_ROWS * K; i += OZ_THREADS) {
      const int r = i % OZ_ROWS, k = i / OZ_ROWS;
      if (r < rows) {
        const float hi = V[(size_t)(r0 + r) + (size_t)(a0 + k) * ldv].x;
        const int E = (int)((__float_as_uint(hi) >> 23) & 0xFFu);
        if (E) atomicMax(&erow[r], E);
      }
    }
    __syncthreads();
    // 2. slices of the tile (padding rows and columns are zero)
    for (int i = tid; i < OZ_ROWS * kp; i += OZ_THREADS) {
      const int r = i % OZ_ROWS, k = i / OZ_ROWS;
      long long x = 0;
      if (r < rows && k < K && erow[r]) {
        const float2 v = V[(size_t)(r0 + r) + (size_t)(a0 + k) * ldv];
        const int e = erow[r] - 126;  // 2^(E-127) <= |hi| < 2^(E-126)
        x = oz_fix56(v.x, e) + oz_fix56(v.y, e);
      }
      const bool neg = x < 0;
      const unsigned long long a = neg ? (unsigned long long)(-x) : (unsigned long long)x;
      for (int s = 0; s < OZ_SA; ++s) {
        const int sl = (int)((a >> (49 - 7 * s)) & 127ull);
        As[((size_t)s * OZ_ROWS + r) * lda + k] = __float2bfloat16_rn(neg ? -(float)sl : (float)sl);
      }
    }
    __syncthreads();
    // 3. output columns in chunks of 32
    for (int c0 = 0; c0 < N; c0 += OZ_NC) {
      // B slices of the chunk, 16-byte copies (kp is a multiple of 16, so rows are 32-byte multiples)
      const int kv = kp / 8;  // uint4 per row
      for (int i = tid; i < OZ_S * OZ_NC * kv; i += OZ_THREADS) {
        const int q = i % kv, cr = (i / kv) % OZ_NC, t = i / (kv * OZ_NC);
        const uint4 w = *reinterpret_cast<const uint4 *>(Bsl + ((size_t)t * np + c0 + cr) * kp + q * 8);
        *reinterpret_cast<uint4 *>(Bs + ((size_t)t * OZ_NC + cr) * ldb + q * 8) = w;
      }
      __syncthreads();
      float acc[2][OZ_L][4];
#pragma unroll
      for (int nt = 0; nt < 2; ++nt)
#pragma unroll
        for (int L = 0; L < OZ_L; ++L)
#pragma unroll
          for (int i = 0; i < 4; ++i) acc[nt][L][i] = 0.0f;
      const int arow = rg * 16 + g;
      for (int k0 = 0; k0 < kp; k0 += 16) {
        unsigned af[OZ_SA][4];
#pragma unroll
        for (int s = 0; s < OZ_SA; ++s) {
          const __nv_bfloat16 *base = As + ((size_t)s * OZ_ROWS + arow) * lda + k0 + 2 * tq;
          af[s][0] = *reinterpret_cast<const unsigned *>(base);
          af[s][1] = *reinterpret_cast<const unsigned *>(base + 8 * lda);
          af[s][2] = *reinterpret_cast<const unsigned *>(base + 8);
          af[s][3] = *reinterpret_cast<const unsigned *>(base + 8 * lda + 8);
        }
#pragma unroll
        for (int nt = 0; nt < 2; ++nt) {
          const int bcol = (half * 2 + nt) * 8 + g;
          unsigned bf[OZ_S][2];
#pragma unroll
          for (int t = 0; t < OZ_S; ++t) {
            const __nv_bfloat16 *base = Bs + ((size_t)t * OZ_NC + bcol) * ldb + k0 + 2 * tq;
            bf[t][0] = *reinterpret_cast<const unsigned *>(base);
            bf[t][1] = *reinterpret_cast<const unsigned *>(base + 8);
          }
#pragma unroll
          for (int s = 0; s < OZ_SA; ++s)
#pragma unroll
            for (int t = 0; t < OZ_S && s + t < OZ_L; ++t) oz_mma(acc[nt][s + t], af[s], bf[t]);
        }
      }
      // recombine the levels exactly as pairs, scale by 2^(e_r + f_c - 7(L+2)) and store
#pragma unroll
      for (int nt = 0; nt < 2; ++nt)
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const int r = arow + ((i & 2) ? 8 : 0);
          const int c = c0 + (half * 2 + nt) * 8 + 2 * tq + (i & 1);
          if (r < rows && c < N && erow[r]) {
            float sh = 0.0f, sl = 0.0f;
#pragma unroll
            for (int L = OZ_L - 1; L >= 0; --L) oz_add(sh, sl, ldexpf(acc[nt][L][i], -7 * (L + 2)));
            const float hi = sh + sl;
            const float lo = sl - (hi - sh);
            const int sc = (erow[r] - 126) + fcol[c];
            V[(size_t)(r0 + r) + (size_t)(s0 + c) * ldv] = make_float2(ldexpf(hi, sc), ldexpf(lo, sc));
          } else if (r < rows && c < N) {
            V[(size_t)(r0 + r) + (size_t)(s0 + c) * ldv] = make_float2(0.0f, 0.0f);  // an all-zero row
          }
        }
      __syncthreads();  // Bs is reloaded for the next chunk
    }
  }
}

// ---------------------------------------------------------------------------------------------------------------
// The same product on the 5th-generation tensor cores: tcgen05.mma (kind::f16, bf16 x bf16 -> FP32) issued by one
// thread, operands in shared memory in the canonical K-major core-matrix layout (8 rows x 16 bytes per core
// matrix, no swizzle), the eight level sums accumulated in TMEM (8 levels x 64 columns = all 512 columns of the
// SM's tensor memory, 128 lanes = the 128 rows of a tile).  Every level sum is exact in FP32, so the result is
// bit-identical to k_restart_tc's whatever the summation order.
//
// Per tile of 128 rows: the row exponents, then all slices of the tile into this CTA's scratch in global memory
// (L2-resident, 2 KB per K column), so that the output chunks -- which overwrite V in place -- never read a
// column that an earlier chunk already wrote.  Per chunk of 64 output columns: K in stages of 32 (two MMA K-steps),
// double-buffered in shared memory and filled by bulk copies of the TMA engine (cp.async.bulk, completion counted
// in bytes on the stage's "full" mbarrier).  One thread runs the pipeline: the copies of stage i+1 are in flight
// while the tensor cores run the 35 MMAs per K-step of stage i; tcgen05.commit arrives on the stage's "empty"
// mbarrier when the MMAs that read it are done.  The epilogue reads TMEM with tcgen05.ld and recombines the levels
// (as pairs, or for FP64 storage as exact integers scaled into one FP64 fused multiply-add).
// ---------------------------------------------------------------------------------------------------------------
constexpr int T5_M = 128;                                  // rows per tile (MMA M)
constexpr int T5_NC = 64;                                  // output columns per chunk (MMA N <= 64)
constexpr int T5_KC = 32;                                  // K per shared-memory stage
constexpr int T5_THREADS = 512;                            // 16 warps: 4 tensor warps, 12 slicing warps
constexpr int T5_ASL = T5_M * T5_KC * 2;                   // bytes of one V slice in a stage
constexpr int T5_BSL = T5_NC * T5_KC * 2;                  // bytes of one Q slice in a stage
constexpr int T5_STAGE = OZ_SA * T5_ASL + OZ_QMAX * T5_BSL;  // 98304
constexpr uint32_t T5_TMEM_COLS = OZ_L * T5_NC;            // 512
// Basis storage of the tcgen05 restart.  T5Pair: FP32 pairs (hi, lo); the row exponent comes from hi, the fixed
// point is the sum of both parts', and the result is written back as a pair.  T5F64: IEEE doubles; the fixed point
// holds the 53-bit significand (truncated only below 2^-56 of the row maximum), and the result is the exact level
// sum rounded once to a double.  Both keep 8 bytes per entry, so the V tile and its copies are the same.
struct T5Pair {
  using T = float2;
  static KS_DEVICE int expo(float2 v) { return (int)((__float_as_uint(v.x) >> 23) & 0xFFu); }
  static KS_DEVICE int escale(int E) { return E - 126; }  // 2^(E-127) <= |hi| < 2^(E-126)
  static KS_DEVICE long long fix56(float2 v, int e) { return oz_fix56(v.x, e) + oz_fix56(v.y, e); }
};
struct T5F64 {
  using T = double;
  static KS_DEVICE int expo(double v) { return (int)((__double_as_longlong(v) >> 52) & 0x7FF); }
  static KS_DEVICE int escale(int E) { return E - 1022; }  // 2^(E-1023) <= |v| < 2^(E-1022)
  // signed 56-bit fixed point of v * 2^(56 - e), |v| < 2^e (so the shift is at most 3); zero for zeros and
  // subnormals, truncated toward zero below 2^-56 of the row maximum
  static KS_DEVICE long long fix56(double v, int e) {
    const unsigned long long u = (unsigned long long)__double_as_longlong(v);
    const int E = (int)((u >> 52) & 0x7FF);
    if (E == 0) return 0;
    const long long m = (long long)((u & 0xFFFFFFFFFFFFFull) | 0x10000000000000ull);
    const int sh = (E - 1075) + 56 - e;
    long long r;
    if (sh >= 0) r = sh <= 3 ? (m << sh) : 0;
    else r = sh > -60 ? (m >> (-sh)) : 0;
    return (u >> 63) ? -r : r;
  }
};

// ---------------------------------------------------------------------------------------------------------------
// The kernel is warp-specialised, so that the phases of consecutive tiles overlap:
//   warps 0-7, the tensor warps: thread 0 runs a chunk's operand-stage pipeline and MMAs (as above) and commits to
//     tmem_full; the eight warps then read the level sums out of TMEM (warp w: lanes 32 (w mod 4) .. +31, every
//     other 16-column group from 16 (w / 4)) and write the outputs.
//   warps 8-15, the slicing warps (256 threads): the row exponents and slices of the CTA's next tile, read from V
//     in global memory and written to the CTA's scratch buffer (tile j in buffer j mod 2), while the tensor warps
//     run the tile before it.
// Hand-offs by mbarriers: ready[b] completes when the 256 slicing threads have filled buffer b (slices and row
// exponents); done[b] when the eight tensor warps have written back the tile of buffer b, so that the tile after
// next may replace it.  Named barriers (1: tensor warps, 2: slicing warps) order each group's own phases.  The
// slicing warps read rows of later tiles than the ones the tensor warps write, and a tile's rows are all read (its
// slices complete) before its own outputs are written, so the in-place update stays safe.  Every wait is bounded;
// a timeout in either group ends both (the other group's next wait runs out), the MMA thread then waits (bounded)
// for its copies and MMAs in flight, and the kernel frees its TMEM and sets *err.
// ---------------------------------------------------------------------------------------------------------------
constexpr int T5W_TENSOR = 256;                       // threads of the tensor warps
constexpr int T5W_SLICERS = T5_THREADS - T5W_TENSOR;  // 256
constexpr int T5W_H = T5W_SLICERS / T5_M;             // slicing threads per row in the exponent pass
constexpr size_t T5W_SMEM = 2 * (size_t)T5_STAGE + (2 + T5W_H) * T5_M * sizeof(int) +
                            9 * sizeof(unsigned long long) + 16 + T5_NC * sizeof(int);

KS_DEVICE void t5_bar(int id, int count) { asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(count) : "memory"); }

// named barrier that also ANDs a flag over the participating threads
KS_DEVICE int t5_bar_and(int id, int count, int v) {
  uint32_t out;
  asm volatile(
      "{\n\t.reg .pred p, q;\n\tsetp.ne.u32 p, %1, 0;\n\tbar.red.and.pred q, %2, %3, p;\n\tselp.u32 %0, 1, 0, q;\n\t}\n"
      : "=r"(out)
      : "r"((uint32_t)v), "r"(id), "r"(count)
      : "memory");
  return (int)out;
}

KS_DEVICE void t5_arrive(unsigned long long *bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(t5_smem(bar)) : "memory");
}

// bounded wait that suspends the warp (up to 500 ns per try) instead of polling, so that waiting warps leave the
// issue slots of their sub-partition to the working ones; a timeout, or another thread's, sets *abort and ends it.
// With abort null the wait runs to its own bound (the MMA thread's waits for copies and MMAs in flight).
KS_DEVICE bool t5w_wait(unsigned long long *bar, uint32_t parity, volatile int *abort) {
  const uint32_t a = t5_smem(bar);
  for (int it = 0; it < T5_WAIT_LIMIT / 16; ++it) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\tselp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(done)
        : "r"(a), "r"(parity), "r"(500u)
        : "memory");
    if (done) return true;
    if ((it & 15) == 15 && abort && *abort) return false;
  }
  if (abort) *abort = 1;
  return false;
}

template <class S, int QS>
__global__ void __launch_bounds__(T5_THREADS, 1)
    k_restart_t5w(typename S::T *__restrict__ V, long long ldv, int n, int a0, int K, int s0, int N, int kp, int np,
                  const __nv_bfloat16 *__restrict__ Bsl, const int *__restrict__ fcol,
                  __nv_bfloat16 *__restrict__ Ascr, int *__restrict__ err, signed char *__restrict__ vexp, int ldt) {
  using T = typename S::T;
  extern __shared__ __align__(1024) unsigned char sm[];
  int *erow = reinterpret_cast<int *>(sm + 2 * T5_STAGE);  // [2][128]: row exponents of the tile in buffer b
  int *etmp = erow + 2 * T5_M;                             // [T5W_H][128]: partial maxima
  unsigned long long *full = reinterpret_cast<unsigned long long *>(etmp + T5W_H * T5_M);  // stage loaded
  unsigned long long *empty = full + 2;                                                     // stage consumed
  unsigned long long *tfull = empty + 2;   // a chunk's MMAs done
  unsigned long long *ready = tfull + 1;   // [2] a tile's slices in buffer b
  unsigned long long *done = ready + 2;    // [2] buffer b's tile written back
  uint32_t *tslot = reinterpret_cast<uint32_t *>(done + 2);
  volatile int *abortf = reinterpret_cast<volatile int *>(tslot + 1);  // a wait of this CTA timed out
  int *cmax = reinterpret_cast<int *>(tslot + 4);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (tid < T5_NC) cmax[tid] = 0;
  if (tid == 0) *abortf = 0;
  const int nk8 = kp / 8;
  const int nkc = (kp + T5_KC - 1) / T5_KC;
  const size_t abuf = (size_t)OZ_SA * nk8 * 16 * 64;       // bf16 elements of one slice buffer
  __nv_bfloat16 *As0 = Ascr + (size_t)blockIdx.x * 2 * abuf;
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(t5_smem(tslot)),
                 "r"(T5_TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    for (int b = 0; b < 2; ++b) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(t5_smem(&full[b])) : "memory");
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(t5_smem(&empty[b])) : "memory");
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(t5_smem(&ready[b])), "r"(T5W_SLICERS) : "memory");
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(t5_smem(&done[b])), "r"(T5W_TENSOR / 32)
                   : "memory");
    }
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(t5_smem(tfull)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  t5_fence_before();
  __syncthreads();
  t5_fence_after();
  const uint32_t tbase = *tslot;
  const int ntiles = (n + T5_M - 1) / T5_M;
  int ok = 1;
  if (warp < T5W_TENSOR / 32) {
    // ---- tensor warps ----
    uint32_t fph[2] = {0u, 0u}, eph[2] = {0u, 0u};  // thread 0: barrier phases and outstanding completions
    int epend[2] = {0, 0}, fpend[2] = {0, 0};
    uint32_t tph = 0u;
    const uint32_t idesc_m = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(T5_M >> 4) << 24);
    int j = 0;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++j) {
      const int b = j & 1;
      const int r0 = tile * T5_M;
      const int rows = min(T5_M, n - r0);
      if (!t5w_wait(&ready[b], (uint32_t)((j >> 1) & 1), abortf)) ok = 0;
      ok = t5_bar_and(1, T5W_TENSOR, ok);
      if (!ok) break;
      const __nv_bfloat16 *As = As0 + (size_t)b * abuf;
      const int *er_b = erow + b * T5_M;
      for (int c0 = 0; c0 < N && ok; c0 += T5_NC) {
        const int nch = min(T5_NC, (N - c0 + 15) / 16 * 16);
        if (tid == 0) {
          const uint32_t idesc = idesc_m | ((uint32_t)(nch >> 3) << 17);
          uint32_t initmask = 0;  // levels already written in this chunk
          auto load = [&](int i) {  // stage i into buffer i & 1, once the MMAs that read the buffer are done
            const int sb = i & 1;
            if (epend[sb]) {
              if (!t5w_wait(&empty[sb], eph[sb], abortf)) {
                ok = 0;  // the buffer may still be read: issue nothing
                return;
              }
              eph[sb] ^= 1u;
              epend[sb] = 0;
            }
            const int kc8 = i * (T5_KC / 8);
            const int sk8 = min(T5_KC / 8, nk8 - kc8);
            unsigned char *st = sm + sb * T5_STAGE;
            const uint32_t abytes = sk8 * 16 * 128, bbytes = (nch / 8) * 128;
            t5_expect_tx(&full[sb], OZ_SA * abytes + QS * sk8 * bbytes);
            for (int sl = 0; sl < OZ_SA; ++sl)
              t5_bulk(st + sl * T5_ASL, As + ((size_t)sl * nk8 + kc8) * 16 * 64, abytes, &full[sb]);
            for (int t = 0; t < QS; ++t)
              for (int k8 = 0; k8 < sk8; ++k8)
                t5_bulk(st + OZ_SA * T5_ASL + t * T5_BSL + k8 * (T5_NC / 8) * 128,
                        Bsl + (((size_t)t * nk8 + kc8 + k8) * (np / 8) + c0 / 8) * 64, bbytes, &full[sb]);
            fpend[sb] = 1;
          };
          load(0);
          for (int i = 0; i < nkc && ok; ++i) {
            const int sb = i & 1;
            if (!t5w_wait(&full[sb], fph[sb], abortf)) {
              ok = 0;
              break;
            }
            fph[sb] ^= 1u;
            fpend[sb] = 0;
            t5_fence_after();
            const int sk8 = min(T5_KC / 8, nk8 - i * (T5_KC / 8));
            const uint32_t abase = t5_smem(sm + sb * T5_STAGE), bbase = abase + OZ_SA * T5_ASL;
            const uint64_t ad0 = t5_desc(abase, 16 * 128, 128);
            const uint64_t bd0 = t5_desc(bbase, (T5_NC / 8) * 128, 128);
            for (int jj = 0; jj < sk8 / 2; ++jj)
#pragma unroll
              for (int sa = 0; sa < OZ_SA; ++sa)
#pragma unroll
                for (int tb = 0; tb < QS; ++tb) {
                  if (sa + tb >= OZ_L) continue;
                  const int L = sa + tb;
                  const uint64_t ad = ad0 + (uint64_t)((sa * T5_ASL + jj * 2 * (16 * 128)) >> 4);
                  const uint64_t bd = bd0 + (uint64_t)((tb * T5_BSL + jj * 2 * ((T5_NC / 8) * 128)) >> 4);
                  t5_mma(tbase + (uint32_t)(L * T5_NC), ad, bd, idesc, (initmask >> L) & 1u);
                  initmask |= 1u << L;
                }
            t5_commit(&empty[sb]);
            epend[sb] = 1;
            if (i + 1 < nkc) load(i + 1);
          }
          // the chunk's level sums are complete when every MMA issued so far is
          if (ok) t5_commit(tfull);
          for (int sb = 0; sb < 2; ++sb) {
            // every copy and MMA in flight completes before the stage buffers or TMEM are reused or freed
            if (epend[sb]) {
              if (!t5w_wait(&empty[sb], eph[sb], nullptr)) ok = 0;
              eph[sb] ^= 1u;
              epend[sb] = 0;
            }
            if (fpend[sb]) {
              if (!t5w_wait(&full[sb], fph[sb], nullptr)) ok = 0;
              fph[sb] ^= 1u;
              fpend[sb] = 0;
            }
          }
        }
        __syncwarp();
        // thread 0's pipeline state joins the vote: after a failure it committed nothing to tmem_full
        ok = t5_bar_and(1, T5W_TENSOR, ok);
        if (!ok) break;
        if (!t5w_wait(tfull, tph, abortf)) ok = 0;
        tph ^= 1u;
        ok = t5_bar_and(1, T5W_TENSOR, ok);
        if (!ok) break;
        t5_fence_after();
        // epilogue: warp w reads lanes 32 w .. +31 (tile rows), every 16-column group of the chunk
        // tensor warp w reads TMEM lanes 32 (w mod 4) .. +31 (tile rows) and every other 16-column group from
        // 16 (w / 4): two warps per sub-partition share the TMEM latency of the level loads
        const int qd = warp & 3;
        const int m = 32 * qd + lane;
        const int er = er_b[m];
#pragma unroll 1
        for (int col = 16 * (warp >> 2); col < nch; col += 16 * (T5W_TENSOR / 128)) {
          if constexpr (std::is_same<S, T5Pair>::value) {
            float sh[16], sl[16];
#pragma unroll
            for (int i2 = 0; i2 < 16; ++i2) sh[i2] = sl[i2] = 0.0f;
#pragma unroll 1
            for (int L = OZ_L - 1; L >= 0; --L) {
              float v[16];
              t5_ld16(tbase + ((uint32_t)(32 * qd) << 16) + (uint32_t)(L * T5_NC + col), v);
              const float scale = __uint_as_float((uint32_t)(127 - 7 * (L + 2)) << 23);
#pragma unroll
              for (int i2 = 0; i2 < 16; ++i2) oz_add(sh[i2], sl[i2], v[i2] * scale);
            }
            if (m < rows) {
#pragma unroll
              for (int i2 = 0; i2 < 16; ++i2) {
                const int c = c0 + col + i2;
                if (c >= N) break;
                float2 out = make_float2(0.0f, 0.0f);  // an all-zero row stays zero
                if (er) {
                  const float hi = sh[i2] + sl[i2];
                  const float lo = sl[i2] - (hi - sh[i2]);
                  const int sc = S::escale(er) + fcol[c];
                  out = make_float2(ldexpf(hi, sc), ldexpf(lo, sc));
                }
                __stcs(V + (size_t)(r0 + m) + (size_t)(s0 + c) * ldv, out);  // streamed out (evict-first)
              }
            }
          } else {
            long long Hs[16], Rs[16];
#pragma unroll
            for (int i2 = 0; i2 < 16; ++i2) Hs[i2] = Rs[i2] = 0;
#pragma unroll 1
            for (int L = OZ_L - 1; L >= 0; --L) {
              float v[16];
              t5_ld16(tbase + ((uint32_t)(32 * qd) << 16) + (uint32_t)(L * T5_NC + col), v);
              const long long w = L >= 2 ? (1ll << (7 * (7 - L))) : (L == 1 ? 1ll : 128ll);
#pragma unroll
              for (int i2 = 0; i2 < 16; ++i2) {
                const long long pl = (long long)__float2int_rn(v[i2]);  // an integer below 2^24 in magnitude
                if (L >= 2) Rs[i2] += pl * w;
                else Hs[i2] += pl * w;
              }
            }
            int ex[16];
#pragma unroll
            for (int i2 = 0; i2 < 16; ++i2) ex[i2] = 0;
            if (m < rows) {
#pragma unroll
              for (int i2 = 0; i2 < 16; ++i2) {
                const int c = c0 + col + i2;
                if (c >= N) break;
                double out = 0.0;  // an all-zero row stays zero
                if (er) {
                  const int sc = S::escale(er) + fcol[c] - 63;
                  out = fma((double)Hs[i2], t5_pow2(sc + 42), (double)Rs[i2] * t5_pow2(sc));
                }
                __stcs(V + (size_t)(r0 + m) + (size_t)(s0 + c) * ldv, out);  // streamed out (evict-first)
                ex[i2] = (int)(((unsigned long long)__double_as_longlong(out) >> 52) & 0x7FF);
              }
            }
            if (vexp) {
#pragma unroll
              for (int i2 = 0; i2 < 16; ++i2) {
                int x = ex[i2];
#pragma unroll
                for (int off = 16; off > 0; off >>= 1) x = max(x, __shfl_xor_sync(0xffffffffu, x, off));
                if (lane == 0 && x) atomicMax(&cmax[col + i2], x);
              }
            }
          }
        }
        t5_fence_before();
        t5_bar(1, T5W_TENSOR);  // TMEM is read out before the next chunk's MMAs overwrite it
        if (vexp) {
          if (tid < nch) {
            // the exponent of each output column over this tile: |v| < 2^(E - 1022), -128 for an all-zero tile
            const int c = c0 + tid;
            if (c < N) {
              const int E = cmax[tid];
              const int e = E == 0 ? -128 : (E - 1022 < -127 ? -127 : (E - 1022 > 127 ? 127 : E - 1022));
              vexp[(size_t)(s0 + c) * ldt + tile] = (signed char)e;
            }
            cmax[tid] = 0;
          }
          t5_bar(1, T5W_TENSOR);
        }
      }
      if (!ok) break;
      // the tile is written back: its buffer may take the tile after next
      __syncwarp();
      if (lane == 0) t5_arrive(&done[b]);
    }
  } else {
    // ---- slicing warps ----
    const int st = tid - T5W_TENSOR;
    int j = 0;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++j) {
      const int b = j & 1;
      const int r0 = tile * T5_M;
      const int rows = min(T5_M, n - r0);
      if (j >= 2 && !t5w_wait(&done[b], (uint32_t)(((j - 2) >> 1) & 1), abortf)) ok = 0;
      ok = t5_bar_and(2, T5W_SLICERS, ok);
      if (!ok) break;
      int *er_b = erow + b * T5_M;
      // 1. row exponents: e_r = 1 + floor(log2 max_k |v|) from the exponent fields (T5W_H threads per row; eight
      //    loads in flight per thread: this pass is the tile's first touch of V)
      {
        const int m = st & (T5_M - 1), h = st >> 7;
        int E = 0;
        if (m < rows)
          for (int k0 = h; k0 < K; k0 += 8 * T5W_H) {
            T vv[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) {
              const int k = k0 + u * T5W_H;
              vv[u] = k < K ? V[(size_t)(r0 + m) + (size_t)(a0 + k) * ldv] : T{};
            }
#pragma unroll
            for (int u = 0; u < 8; ++u) E = max(E, S::expo(vv[u]));
          }
        etmp[h * T5_M + m] = E;
        t5_bar(2, T5W_SLICERS);
        if (h == 0) {
#pragma unroll
          for (int q = 1; q < T5W_H; ++q) E = max(E, etmp[q * T5_M + m]);
          er_b[m] = E;
        }
        t5_bar(2, T5W_SLICERS);
      }
      // the CTA's next tile into L2 while this one is sliced (one 128-byte line per 16 rows and column)
      {
        const int rn = r0 + (int)gridDim.x * T5_M;
        if (rn < n)
          for (int q = st; q < K * 8; q += T5W_SLICERS) {
            const int r = rn + 16 * (q & 7);
            if (r < n) asm volatile("prefetch.global.L2 [%0];" ::"l"(V + (size_t)r + (size_t)(a0 + (q >> 3)) * ldv));
          }
      }
      // 2. all slices of the tile into buffer b, one core-matrix row (8 consecutive k of one row) per item, two
      //    items per pass (32 consecutive rows per warp: every load of a column is one coalesced 256-byte access)
      __nv_bfloat16 *As = As0 + (size_t)b * abuf;
      for (int it0 = st; it0 < T5_M * nk8; it0 += 2 * T5W_SLICERS) {
        T v[2][8];
#pragma unroll
        for (int p2 = 0; p2 < 2; ++p2) {
          const int it = it0 + p2 * T5W_SLICERS;
          const int m = it & (T5_M - 1), k8 = it >> 7;
#pragma unroll
          for (int jj = 0; jj < 8; ++jj) {
            const int k = 8 * k8 + jj;
            // the tile's second and last read of V: evict-first, so the slice scratch keeps its L2 lines
            v[p2][jj] = (it < T5_M * nk8 && m < rows && k < K) ? __ldcs(V + (size_t)(r0 + m) + (size_t)(a0 + k) * ldv)
                                                               : T{};
          }
        }
#pragma unroll
        for (int p2 = 0; p2 < 2; ++p2) {
          const int it = it0 + p2 * T5W_SLICERS;
          if (it >= T5_M * nk8) break;
          const int m = it & (T5_M - 1), k8 = it >> 7;
          const int er = er_b[m];
          uint32_t mh[8], ml[8], ng[8];
#pragma unroll
          for (int jj = 0; jj < 8; ++jj) {
            long long x = 0;
            if (er) x = S::fix56(v[p2][jj], S::escale(er));
            ng[jj] = x < 0 ? 1u : 0u;
            const unsigned long long a = x < 0 ? (unsigned long long)(-x) : (unsigned long long)x;
            mh[jj] = (uint32_t)(a >> 32);
            ml[jj] = (uint32_t)a;
          }
#pragma unroll
          for (int sl = 0; sl < OZ_SA; ++sl) {
            uint32_t u[8];
#pragma unroll
            for (int jj = 0; jj < 8; ++jj) u[jj] = t5_field(mh[jj], ml[jj], sl);
            uint4 w;
            w.x = t5_slice_pair(u[0], u[1], ng[0], ng[1]);
            w.y = t5_slice_pair(u[2], u[3], ng[2], ng[3]);
            w.z = t5_slice_pair(u[4], u[5], ng[4], ng[5]);
            w.w = t5_slice_pair(u[6], u[7], ng[6], ng[7]);
            *reinterpret_cast<uint4 *>(As + (((size_t)sl * nk8 + k8) * 16 + (m >> 3)) * 64 + (m & 7) * 8) = w;
          }
        }
      }
      // the TMA engine reads the buffer next (async proxy): order this thread's writes before the hand-off
      asm volatile("fence.proxy.async;" ::: "memory");
      t5_arrive(&ready[b]);
    }
  }
  t5_fence_before();
  const int bad = __syncthreads_or(!ok);
  t5_fence_after();
  if (bad && tid == 0) atomicExch(err, 1);
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tbase), "r"(T5_TMEM_COLS) : "memory");
}

// scratch of the tcgen05 restart: the Q slices (as for k_restart_tc), then per CTA the V slices of a tile
// (OZ_SA x ldp x 128 bf16), then the timeout flag
static size_t t5_qbytes(int ld) { return (restart_tc_scratch_bytes(ld) + 255) / 256 * 256; }
static size_t t5_abytes(int ld) {
  const int ldp = (ld + 15) / 16 * 16;
  return (size_t)num_sms() * 2 * OZ_SA * ldp * 128 * sizeof(__nv_bfloat16);  // two buffers per CTA
}
size_t restart_t5_scratch_bytes(int ld) { return t5_qbytes(ld) + t5_abytes(ld) + 256; }
int *restart_t5_errflag(void *scratch, int ld) {
  return reinterpret_cast<int *>(static_cast<unsigned char *>(scratch) + t5_qbytes(ld) + t5_abytes(ld));
}

template <class S, int QS>
static cudaError_t restart_t5_go(typename S::T *V, long long ldv, int n, int a0, int K, int s0, int N,
                                 const double *Q, int ldq, void *scratch, int ld, cudaStream_t s,
                                 signed char *vexp = nullptr, int ldt = 0) {
  if (N <= 0 || K <= 0) return cudaSuccess;
  if (K > ld || N > ld) return cudaErrorInvalidValue;
  const int kp = (K + 15) / 16 * 16;
  const int ldp = (ld + 15) / 16 * 16;
  const int np = (ld + OZ_NC - 1) / OZ_NC * OZ_NC;
  if (kp > ldp || np < (N + 15) / 16 * 16) return cudaErrorInvalidValue;
  if ((size_t)K * T5_M * 8 > 2 * (size_t)T5_STAGE) return cudaErrorInvalidValue;  // the V tile's room
  // level sums exact in FP32: at most min(QS, 8) products of magnitude <= 127 * 128 per level and k
  if ((long long)(QS > OZ_L ? OZ_L : QS) * 127 * 128 * kp >= (1ll << 24)) return cudaErrorInvalidValue;
  __nv_bfloat16 *B = static_cast<__nv_bfloat16 *>(scratch);
  int *fcol = reinterpret_cast<int *>(B + (size_t)OZ_QMAX * np * kp);
  __nv_bfloat16 *Ascr = reinterpret_cast<__nv_bfloat16 *>(static_cast<unsigned char *>(scratch) + t5_qbytes(ld));
  int *err = restart_t5_errflag(scratch, ld);
  cudaError_t e = cudaFuncSetAttribute(k_restart_t5w<S, QS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)T5W_SMEM);
  if (e != cudaSuccess) return e;
  k_oz_qslice<<<np, 128, 0, s>>>(Q, ldq, a0, s0, K, N, kp, np, B, fcol, 1, QS);
  const int ntiles = (n + T5_M - 1) / T5_M;
  int blocks = num_sms();
  if (blocks > ntiles) blocks = ntiles;
  k_restart_t5w<S, QS><<<blocks, T5_THREADS, T5W_SMEM, s>>>(V, ldv, n, a0, K, s0, N, kp, np, B, fcol, Ascr, err,
                                                            vexp, ldt);
  return cudaGetLastError();
}

cudaError_t launch_restart_t5(float2 *V, long long ldv, int n, int a0, int K, int s0, int N, const double *Q, int ldq,
                              void *scratch, int ld, cudaStream_t s) {
  return restart_t5_go<T5Pair, OZ_S>(V, ldv, n, a0, K, s0, N, Q, ldq, scratch, ld, s);
}

// FP64 storage: Q in 8 slices (56 bits) while the level sums stay exact (K <= 128), else 7
cudaError_t launch_restart_t5_f64(double *V, long long ldv, int n, int a0, int K, int s0, int N, const double *Q,
                                  int ldq, void *scratch, int ld, cudaStream_t s, signed char *vexp, int ldt) {
  if ((K + 15) / 16 * 16 <= 128)
    return restart_t5_go<T5F64, OZ_QMAX>(V, ldv, n, a0, K, s0, N, Q, ldq, scratch, ld, s, vexp, ldt);
  return restart_t5_go<T5F64, OZ_S>(V, ldv, n, a0, K, s0, N, Q, ldq, scratch, ld, s, vexp, ldt);
}

cudaError_t launch_restart_tc(float2 *V, long long ldv, int n, int a0, int K, int s0, int N, const double *Q, int ldq,
                              void *scratch, int ld, cudaStream_t s) {
  if (N <= 0 || K <= 0) return cudaSuccess;
  if (K > ld || N > ld) return cudaErrorInvalidValue;
  const int kp = (K + 15) / 16 * 16;
  const int ldp = (ld + 15) / 16 * 16;
  const int np = (ld + OZ_NC - 1) / OZ_NC * OZ_NC;  // layout of the scratch (fixed per EPS)
  if (kp > ldp) return cudaErrorInvalidValue;
  __nv_bfloat16 *B = static_cast<__nv_bfloat16 *>(scratch);
  int *fcol = reinterpret_cast<int *>(B + (size_t)OZ_QMAX * np * kp);
  const size_t shm = oz_smem_bytes(kp);
  if (shm > (size_t)227 * 1024) return cudaErrorInvalidValue;
  cudaError_t err = cudaFuncSetAttribute(k_restart_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm);
  if (err != cudaSuccess) return err;
  k_oz_qslice<<<np, 128, 0, s>>>(Q, ldq, a0, s0, K, N, kp, np, B, fcol, 0, OZ_S);
  const int ntiles = (n + OZ_ROWS - 1) / OZ_ROWS;
  int blocks = num_sms();
  if (blocks > ntiles) blocks = ntiles;
  k_restart_tc<<<blocks, OZ_THREADS, shm, s>>>(V, ldv, n, a0, K, s0, N, kp, np, B, fcol);
  return cudaGetLastError();
}

}  // namespace ksg
