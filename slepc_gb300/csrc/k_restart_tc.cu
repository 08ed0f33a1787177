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

#include "common.cuh"
#include "kernels.h"
#include "ks_types.h"

namespace ksg {

constexpr int OZ_SA = 8;         // slices of V (56 bits)
constexpr int OZ_S = 7;          // slices of Q (49 bits)
constexpr int OZ_L = 8;          // levels s + t kept
constexpr int OZ_ROWS = 64;      // rows of V per tile
constexpr int OZ_THREADS = 256;  // 8 warps: 4 row groups of 16 x 2 column halves of a chunk
constexpr int OZ_NC = 32;        // output columns per chunk (4 mma n-tiles)
constexpr int OZ_PAD = 8;        // bf16 padding per row of the Q slices (rows stay 16-byte aligned for 16-byte copies)
constexpr int OZ_PADA = 2;       // bf16 padding per row of the V slices: an odd word stride, so the slicing pass's
                                 // stores from 32 consecutive rows hit 32 banks

size_t restart_tc_scratch_bytes(int ld) {
  const int kp = (ld + 15) / 16 * 16, np = (ld + OZ_NC - 1) / OZ_NC * OZ_NC;
  return (size_t)OZ_S * np * kp * sizeof(__nv_bfloat16) + (size_t)np * sizeof(int) + 256;
}

static size_t oz_smem_bytes(int kp) {
  return ((size_t)OZ_SA * OZ_ROWS * (kp + OZ_PADA) + (size_t)OZ_S * OZ_NC * (kp + OZ_PAD)) *
             sizeof(__nv_bfloat16) +
         OZ_ROWS * sizeof(int) + 16;
}

// Column exponents and slices of Q(a0 + k, s0 + c), k < K, c < N (zero-padded to kp x np): one block per column.
__global__ void k_oz_qslice(const double *__restrict__ Q, int ldq, int a0, int s0, int K, int N, int kp, int np,
                            __nv_bfloat16 *__restrict__ B, int *__restrict__ fcol) {
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
  for (int k = threadIdx.x; k < kp; k += blockDim.x) {
    long long y = 0;
    if (col_ok && k < K) y = __double2ll_rn(scalbn(Q[(a0 + k) + (size_t)(s0 + c) * ldq], 49 - f));
    const bool neg = y < 0;
    const unsigned long long a = neg ? (unsigned long long)(-y) : (unsigned long long)y;
    for (int t = 0; t < OZ_S; ++t) {
      // 7-bit slices; only the top one may reach 128 (when |q| 2^(49-f) rounds up to 2^49)
      const int sl = (int)((a >> (42 - 7 * t)) & (t == 0 ? 255ull : 127ull));
      B[((size_t)t * np + c) * kp + k] = __float2bfloat16_rn(neg ? -(float)sl : (float)sl);
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

cudaError_t launch_restart_tc(float2 *V, long long ldv, int n, int a0, int K, int s0, int N, const double *Q, int ldq,
                              void *scratch, int ld, cudaStream_t s) {
  if (N <= 0 || K <= 0) return cudaSuccess;
  if (K > ld || N > ld) return cudaErrorInvalidValue;
  const int kp = (K + 15) / 16 * 16;
  const int ldp = (ld + 15) / 16 * 16;
  const int np = (ld + OZ_NC - 1) / OZ_NC * OZ_NC;  // layout of the scratch (fixed per EPS)
  if (kp > ldp) return cudaErrorInvalidValue;
  __nv_bfloat16 *B = static_cast<__nv_bfloat16 *>(scratch);
  int *fcol = reinterpret_cast<int *>(B + (size_t)OZ_S * np * kp);
  const size_t shm = oz_smem_bytes(kp);
  if (shm > (size_t)227 * 1024) return cudaErrorInvalidValue;
  cudaError_t err = cudaFuncSetAttribute(k_restart_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm);
  if (err != cudaSuccess) return err;
  k_oz_qslice<<<np, 128, 0, s>>>(Q, ldq, a0, s0, K, N, kp, np, B, fcol);
  const int ntiles = (n + OZ_ROWS - 1) / OZ_ROWS;
  int blocks = num_sms();
  if (blocks > ntiles) blocks = ntiles;
  k_restart_tc<<<blocks, OZ_THREADS, shm, s>>>(V, ldv, n, a0, K, s0, N, kp, np, B, fcol);
  return cudaGetLastError();
}

}  // namespace ksg
