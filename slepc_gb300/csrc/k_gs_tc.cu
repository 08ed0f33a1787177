// k_gs_tc.cu -- the DCGS2 Gram-Schmidt pair for IEEE-double storage on the 16-bit tensor cores (tcgen05 + TMEM), by
// the error-free slice split of Ozaki, Ogita, Oishi and Rump ("Error-free transformations of matrix multiplication
// by using fast routines of matrix multiplication and its applications", Numer. Algorithms 59, 2012).
//
// GB300's FP64 pipe issues about 0.6 T FMA/s, so the FP64-FMA Gram-Schmidt kernels (two FMAs per 8-byte basis
// entry) stop near 2.4 TB/s, a third of the HBM rate.  Here every product runs exactly on the tensor cores:
//
//   a basis value v with |v| < 2^e is the 55-bit two's complement fixed point X = trunc(v 2^(55-e)) (the 53-bit
//   significand truncated only below 2^-55 of the scale), cut into seven bytes B_0 (signed) .. B_6 (unsigned) with
//   X = sum_k B_k 2^(8(6-k)); a vector value u (half A) is cut into eight signed 7-bit slices of its 56-bit fixed
//   point, a coefficient value (half B) into seven bytes like v.  Every slice is an integer below 256 in magnitude,
//   exact in FP16 (the bytes come out of the fixed point's words by byte permutes: FP16(1024 + b) has the bits
//   0x6400 | b, and one exact FP16 subtraction leaves b), every product of two slices is exact, and the tensor
//   cores' FP32 sums of them stay exact below 2^24.
//
// Scales.  Basis columns (unit vectors) carry one exponent per column and 128-row tile, recorded by the kernels that
// write them (this file's update half, the tcgen05 restart) in an int8 table [column][tile]; a value's scale is the
// maximum over the tiles it is summed with, so small entries keep their relative precision where the column is
// small.  u, w (half A) get a scale per row chunk, the coefficient vectors s, g (half B) one per vector, computed on
// the fly.  A value at or above its recorded scale sets the error flag (the host reports PETSC_ERR_PLIB).
//
// Half A (dot): s = V^T u, b = V^T w over chunks of ct <= 4 tiles of 128 rows (|D| <= 512 * 255 * 127 < 2^24).
// MMA M = 128 = 16 basis columns x 8 slice slots (row jl * 8 + k; slot 7 stays zero), N = 16 = 2 vectors x 8
// slices, K = the rows.  The exact chunk sums of one column, recombined by a butterfly over its 8 lanes as a
// 128-bit integer, are rounded once and accumulated across chunks in double-double; the last block merges the block
// partials in block order and runs the DCGS2 coefficient algebra (gs_epilogue).
//
// Half B (update): [v w'] = [(sigma u - V s) / nu, w - V g - tau sigma u].  Per tile of 128 rows: MMA M = 128 rows,
// N = 16 (s, g x 8 byte slots), K = the basis columns, one TMEM accumulator per V byte; the thread of row r sums the
// 13 levels k + q exactly in 32-bit integers and rounds the product once; the FP64 update, the norm of w' and the
// recorded exponents of v follow.  Results are deterministic: fixed partitions, fixed orders, no floating-point
// atomics.
//
// Shared-memory layouts are the canonical K-major core matrices (8 rows x 16 bytes, no swizzle).  In half A the
// core matrices adjacent along K sit 2064 bytes apart instead of 2048, so the slicers' 16-byte stores of one warp
// spread over all bank groups (the unpadded stride put every store of a warp in the same four banks).
//
// Warp roles (13 warps, at most 128 registers each: 4 warps share a sub-partition's 16K registers): 0-3 epilogue
// and vector staging (TMEM lanes 0-127), 4 the MMA issuer (one thread), 5-12 slicers (global loads of V, one stage
// ahead, slicing into a ring of four shared-memory stages).  Stages, B buffers and TMEM buffers hand over on
// mbarriers; tcgen05.commit releases what the tensor cores have read.  Every wait is bounded: on a timeout the
// kernel records it, stops issuing, waits (bounded) for the MMAs in flight, frees TMEM and returns.
#include <cuda_fp16.h>
#include <float.h>

#include <type_traits>

#include "common.cuh"
#include "gs_fixed.cuh"
#include "kernels.h"
#include "krylov_body.cuh"
#include "ks_types.h"
#include "tc_common.cuh"

namespace ksg {

constexpr int GT_R = 128;                                 // rows per tile
constexpr int GT_NA = 4;                                  // A stages (a power of two: slot = q & 3)
constexpr int GT_DLBO = 2064;                             // half A: bytes between core matrices adjacent in K
constexpr int GT_DSTAGE = 16 * GT_DLBO;                   // half A stage: 128 rows of 16 columns (8 slots)
constexpr int GT_USTAGE = 7 * 4096;                       // half B stage: 7 byte matrices of 128 rows x 16 columns
constexpr int GT_STAGE = GT_DSTAGE > GT_USTAGE ? GT_DSTAGE : GT_USTAGE;
constexpr int GT_BLBO = 272;                              // half A B-operand: bytes between core matrices along K
constexpr int GT_BT = 16 * GT_BLBO;                       // half A: u/w slices of one tile
constexpr int GT_CTMAX = 4;                               // tiles per chunk (half A): 512 rows keep sums exact
constexpr int GT_EW = 4, GT_SW = 8;                       // epilogue warps, slicer warps
constexpr int GT_MWARP = GT_EW;                           // the MMA warp
constexpr int GT_SW0 = GT_EW + 1;                         // first slicer warp
constexpr int GT_THREADS = 32 * (GT_EW + 1 + GT_SW);      // 416
constexpr int GT_MAXJ = 144;
constexpr uint32_t GT_TMEM = 512;
// FP16 instruction descriptor: D = FP32, A = B = FP16, both K-major, N = 16, M = 128
constexpr uint32_t GT_IDESC = (1u << 4) | ((uint32_t)(16 >> 3) << 17) | ((uint32_t)(GT_R >> 4) << 24);
// barriers: afull[4] aempty[4] bfull[2] cdone[2] tfree[2] fin
constexpr int GB_AFULL = 0, GB_AEMPTY = 4, GB_BFULL = 8, GB_CDONE = 10, GB_TFREE = 12, GB_FIN = 14, GB_N = 15;

// dynamic shared memory: A ring, then (dot) two chunk B buffers / (update) the coefficient slices, then bookkeeping
constexpr size_t GT_AOFF = 0;
constexpr size_t GT_BOFF = GT_AOFF + (size_t)GT_NA * GT_STAGE;
constexpr size_t GT_DOT_MISC = GT_BOFF + 2 * (size_t)GT_CTMAX * GT_BT;  // dd partials [J][2][2] after the B buffers
constexpr size_t GT_UPD_MISC = GT_BOFF + (size_t)(GT_MAXJ / 8) * 2 * 128;
constexpr size_t GT_MISC_BYTES = (size_t)GT_MAXJ * 4 * 8 + 64 * 8 + GB_N * 8 + 64 * 4 + 16;
constexpr size_t GT_DOT_SMEM = GT_DOT_MISC + GT_MISC_BYTES;
constexpr size_t GT_UPD_SMEM = GT_UPD_MISC + GT_MISC_BYTES;

struct GTShared {
  double *pdd;          // [GT_MAXJ][2 vectors][hi, lo]
  double *red;          // 64 doubles of reduction scratch
  unsigned long long *bar;
  int *ints;            // [0] abort, [1] epilogue-warp barrier counter, [4..7] and [8..11] per-warp maxima,
                        // [12..15] per-tile-slot arrival counters, [16..31] per-tile-slot warp maxima
  uint32_t *tslot;
};

KS_DEVICE GTShared gt_shared(unsigned char *sm, size_t misc) {
  GTShared s;
  s.pdd = reinterpret_cast<double *>(sm + misc);
  s.red = s.pdd + GT_MAXJ * 4;
  s.bar = reinterpret_cast<unsigned long long *>(s.red + 64);
  s.ints = reinterpret_cast<int *>(s.bar + GB_N);
  s.tslot = reinterpret_cast<uint32_t *>(s.ints + 64);
  return s;
}

// Bounded wait that gives up at once when another role has aborted; false on timeout or abort.  Each try suspends
// the thread for up to 0.5 us instead of spinning, so waiting warps leave their issue slots to the slicers; at most
// T5_WAIT_LIMIT / 16 tries.
KS_DEVICE bool gt_wait(unsigned long long *bar, uint32_t parity, volatile int *abort) {
  const uint32_t a = t5_smem(bar);
  for (int it = 0; it < T5_WAIT_LIMIT / 16; ++it) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\tselp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(done)
        : "r"(a), "r"(parity), "r"(500u)
        : "memory");
    if (done) return true;
    if ((it & 15) == 15 && *abort) return false;
  }
  *abort = 1;
  return false;
}

KS_DEVICE void gt_arrive(unsigned long long *bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(t5_smem(bar)) : "memory");
}

KS_DEVICE void gt_fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// Barrier of the four epilogue warps on a shared counter: each warp adds one arrival, then waits (bounded, giving up
// on an abort) until the counter reaches 4 * gen.  Unlike a named barrier it cannot hang when another role has
// stopped early.  Returns false on timeout or abort.
KS_DEVICE bool gt_ebar(int *cnt, int gen, volatile int *abort) {
  __syncwarp();
  __threadfence_block();
  if ((threadIdx.x & 31) == 0) atomicAdd(cnt, 1);
  bool ok = true;
  for (int it = 0;; ++it) {
    if (*(volatile int *)cnt >= GT_EW * gen) break;
    if (it >= T5_WAIT_LIMIT || ((it & 63) == 63 && *abort)) {
      *abort = 1;
      ok = false;
      break;
    }
  }
  __syncwarp();
  __threadfence_block();
  return ok;
}

// 55-bit two's complement fixed point of v relative to 2^e: trunc(v 2^(55-e)); *ovf is set when |v| >= 2^e
KS_DEVICE long long gt_fix55(double v, int e, int *ovf) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(v);
  const int E = (int)((u >> 52) & 0x7FF);
  if (E == 0) return 0;  // zero (or subnormal: below 2^-1022, far below any recorded scale's 2^-55)
  const int sh = (E - 1075) + 55 - e;
  const unsigned long long m = (u & 0xFFFFFFFFFFFFFull) | 0x10000000000000ull;
  if (sh > 2) *ovf = 1;
  const unsigned long long x = sh >= 0 ? (sh <= 2 ? (m << sh) : 0ull) : (sh > -60 ? (m >> (-sh)) : 0ull);
  return (u >> 63) ? -(long long)x : (long long)x;
}

// Seven byte slices of eight fixed points X_0..X_7 (consecutive along K): out[k] = the 16-byte core-matrix row of byte
// B_k (k = 0 the signed top byte) of the eight values, as FP16 integers.  Byte permutes put each byte of two values
// beside the exponent byte 0x64 (FP16(1024 + b) = 0x6400 | b); one exact FP16 subtraction per pair leaves b
// (1152 for the top byte, whose sign bit was flipped to make it 128 + B_0).
KS_DEVICE void gt_bytes7(const long long *X, uint4 *out) {
  const uint32_t C = 0x64646464u;
  const __half2 k1024 = __floats2half2_rn(1024.0f, 1024.0f), k1152 = __floats2half2_rn(1152.0f, 1152.0f);
  uint32_t w[7][4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const uint32_t l0 = (uint32_t)X[2 * i], l1 = (uint32_t)X[2 * i + 1];
    const uint32_t h0 = (uint32_t)((unsigned long long)X[2 * i] >> 32) ^ 0x00800000u;
    const uint32_t h1 = (uint32_t)((unsigned long long)X[2 * i + 1] >> 32) ^ 0x00800000u;
    const uint32_t tl01 = __byte_perm(l0, l1, 0x5140), tl23 = __byte_perm(l0, l1, 0x7362);
    const uint32_t th01 = __byte_perm(h0, h1, 0x5140), th2 = __byte_perm(h0, h1, 0x7362);
    uint32_t r[7];
    r[6] = __byte_perm(tl01, C, 0x5140);  // byte 0 of the low word: B_6
    r[5] = __byte_perm(tl01, C, 0x5342);  // byte 1: B_5
    r[4] = __byte_perm(tl23, C, 0x5140);  // byte 2: B_4
    r[3] = __byte_perm(tl23, C, 0x5342);  // byte 3: B_3
    r[2] = __byte_perm(th01, C, 0x5140);  // high word byte 0: B_2
    r[1] = __byte_perm(th01, C, 0x5342);  // byte 1: B_1
    r[0] = __byte_perm(th2, C, 0x5140);   // byte 2: 128 + B_0
#pragma unroll
    for (int k = 0; k < 7; ++k) {
      __half2 hv = *reinterpret_cast<const __half2 *>(&r[k]);
      hv = __hsub2(hv, k == 0 ? k1152 : k1024);
      w[k][i] = *reinterpret_cast<const uint32_t *>(&hv);
    }
  }
#pragma unroll
  for (int k = 0; k < 7; ++k) out[k] = make_uint4(w[k][0], w[k][1], w[k][2], w[k][3]);
}

// Two signed 7-bit slices as an FP16x2 word: 0x6400 | u is FP16(1024 + u), one exact subtraction leaves u, then the
// sign bits (a negative value's zero slice is -0)
KS_DEVICE uint32_t gt_h_pair(uint32_t u0, uint32_t u1, uint32_t neg0, uint32_t neg1) {
  const uint32_t biased = 0x64006400u | u0 | (u1 << 16);
  const __half2 d = __hsub2(*reinterpret_cast<const __half2 *>(&biased), __floats2half2_rn(1024.0f, 1024.0f));
  return *reinterpret_cast<const uint32_t *>(&d) | (neg0 << 15) | (neg1 << 31);
}

// Eight doubles (consecutive along K) -> eight 7-bit slices (sign and magnitude) of their 56-bit fixed point
// relative to 2^e, as FP16 core-matrix rows; *ovf is set when some |v| >= 2^e.  Used for the vectors u, w of half A.
KS_DEVICE void gt_slice8h(const double *v, int e, uint4 *out, int *ovf) {
  uint32_t mh[8], ml[8], ng[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const unsigned long long u = (unsigned long long)__double_as_longlong(v[j]);
    const int E = (int)((u >> 52) & 0x7FF);
    unsigned long long x = 0;
    if (E) {
      const int sh = (E - 1075) + 56 - e;
      const unsigned long long m = (u & 0xFFFFFFFFFFFFFull) | 0x10000000000000ull;
      if (sh > 3) *ovf = 1;
      x = sh >= 0 ? (sh <= 3 ? (m << sh) : 0ull) : (sh > -60 ? (m >> (-sh)) : 0ull);
    }
    ng[j] = (uint32_t)(u >> 63);
    mh[j] = (uint32_t)(x >> 32);
    ml[j] = (uint32_t)x;
  }
#pragma unroll
  for (int sl = 0; sl < 8; ++sl) {
    uint32_t f[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) f[j] = t5_field(mh[j], ml[j], sl);
    out[sl].x = gt_h_pair(f[0], f[1], ng[0], ng[1]);
    out[sl].y = gt_h_pair(f[2], f[3], ng[2], ng[3]);
    out[sl].z = gt_h_pair(f[4], f[5], ng[4], ng[5]);
    out[sl].w = gt_h_pair(f[6], f[7], ng[6], ng[7]);
  }
}

// (hi, lo) = Y * 2^sh for a signed Y = H 2^42 + R (|H| < 2^33, |R| < 2^61), 0 <= sh < 64
KS_DEVICE void gt_make128(long long H, long long R, int sh, long long &hi, unsigned long long &lo) {
  hi = H >> 22;
  lo = (unsigned long long)H << 42;
  gt_add128(hi, lo, R >> 63, (unsigned long long)R);
  if (sh > 0) {
    hi = (long long)(((unsigned long long)hi << sh) | (lo >> (64 - sh)));
    lo <<= sh;
  }
}
KS_DEVICE void gt_init_barriers(const GTShared &S) {
  const int counts[GB_N] = {GT_SW, GT_SW, GT_SW, GT_SW, 1, 1, 1, 1, GT_EW, GT_EW, 1, 1, GT_EW, GT_EW, 1};
  for (int i = 0; i < GB_N; ++i)
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(t5_smem(&S.bar[i])), "r"(counts[i]) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

KS_DEVICE void gt_load8(const double *col, long long r0, int n, bool valid, double *v) {
  if (valid && r0 + 8 <= n) {
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const double2 d2 = __ldcs(reinterpret_cast<const double2 *>(col) + k);
      v[2 * k] = d2.x;
      v[2 * k + 1] = d2.y;
    }
  } else {
#pragma unroll
    for (int k = 0; k < 8; ++k) v[k] = (valid && r0 + k < n) ? col[k] : 0.0;
  }
}

// ---------------------------------------------------------------------------------------------------------------
// Half A
// ---------------------------------------------------------------------------------------------------------------
template <int NX>
__global__ void __maxnreg__(128) k_gs_dot_tc(StepArgs a, int mode, GTArgs g) {
  KrylovState *st = a.st;
  if (st->stop) return;
  extern __shared__ __align__(1024) unsigned char sm[];
  __shared__ double res[GT_MAXJ * 2 + 4];
  __shared__ int s_last;
  const GTShared S = gt_shared(sm, GT_DOT_MISC);
  volatile int *abort = S.ints;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int n = a.n, J = a.J, NMB = (J + 15) / 16, ct = g.ct;
  const double sigma = st->sigma;
  const double *U = static_cast<const double *>(a.U);
  const double *W = static_cast<const double *>(a.W);
  const double *V = static_cast<const double *>(a.V);
  const int ntiles = (n + GT_R - 1) / GT_R;
  const int nchunks = (ntiles + ct - 1) / ct;
  const int my = blockIdx.x < nchunks ? (nchunks - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
  if (tid == 0) {
    for (int i = 0; i < 64; ++i) S.ints[i] = 0;
    gt_init_barriers(S);
  }
  for (int i = tid; i < GT_MAXJ * 4; i += GT_THREADS) S.pdd[i] = 0.0;
  // slot 7 of every column in the A stages is never written: the whole ring starts at zero
  for (int i = tid; i < GT_NA * GT_STAGE / 16; i += GT_THREADS)
    reinterpret_cast<uint4 *>(sm + GT_AOFF)[i] = make_uint4(0u, 0u, 0u, 0u);
  gt_fence_async_smem();
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(t5_smem(S.tslot)),
                 "r"(GT_TMEM)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  t5_fence_before();
  __syncthreads();
  t5_fence_after();
  const uint32_t tbase = *S.tslot;
  unsigned char *As = sm + GT_AOFF;
  unsigned char *Bs = sm + GT_BOFF;
  double sc0 = 0.0, sc1 = 0.0, sc2 = 0.0;  // u.u, u.w, w.w (epilogue threads)

  if (warp < GT_EW) {
    // ---------------- epilogue warps: u/w staging and TMEM drain ----------------
    const int e = tid;  // 0..127: the 8-row group of a chunk this thread stages, and its TMEM lane
    int ebar_gen = 0;
    int eu0 = 0, ew0 = 0, eu1 = 0, ew1 = 0;  // chunk scales of the two B buffers
    auto stage_uw = [&](int i) -> bool {
      const int b = i & 1;
      const int c = blockIdx.x + i * gridDim.x;
      const long long r0 = (long long)c * ct * GT_R + 8 * e;
      double uv[8], wv[8];
      int Eu = 0, Ew = 0;
      const bool mine = e < ct * 16;
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        const long long r = r0 + k;
        double u = 0.0, w = 0.0;
        if (mine && r < n) {
          u = U[r] * sigma;
          if (NX == 2) w = W[r];
        }
        uv[k] = u;
        wv[k] = w;
        sc0 = fma(u, u, sc0);
        if (NX == 2) {
          sc1 = fma(u, w, sc1);
          sc2 = fma(w, w, sc2);
        }
        Eu = max(Eu, gt_expo(u));
        Ew = max(Ew, gt_expo(w));
      }
      // chunk scales: the largest exponent over the 128 staging threads (every thread keeps its own copy)
      for (int off = 16; off > 0; off >>= 1) {
        Eu = max(Eu, __shfl_xor_sync(0xffffffffu, Eu, off));
        Ew = max(Ew, __shfl_xor_sync(0xffffffffu, Ew, off));
      }
      if (lane == 0) {
        S.ints[4 + warp] = Eu;
        S.ints[8 + warp] = Ew;
      }
      if (!gt_ebar(&S.ints[1], ++ebar_gen, abort)) return false;
      int eu = 0, ew = 0;
#pragma unroll
      for (int q = 0; q < GT_EW; ++q) {
        eu = max(eu, S.ints[4 + q]);
        ew = max(ew, S.ints[8 + q]);
      }
      if (!gt_ebar(&S.ints[1], ++ebar_gen, abort)) return false;  // read by all before the next staging
      eu = gt_escale(eu);
      ew = gt_escale(ew);
      if (b == 0) { eu0 = eu; ew0 = ew; } else { eu1 = eu; ew1 = ew; }
      if (mine) {
        uint4 sl[8];
        int ovf = 0;
        const int t = e >> 4, k8 = e & 15;
        unsigned char *base = Bs + (size_t)b * GT_CTMAX * GT_BT + (size_t)(t * 16 + k8) * GT_BLBO;
        gt_slice8h(uv, eu, sl, &ovf);
#pragma unroll
        for (int q = 0; q < 8; ++q) *reinterpret_cast<uint4 *>(base + q * 16) = sl[q];
        if (NX == 2) gt_slice8h(wv, ew, sl, &ovf);
#pragma unroll
        for (int q = 0; q < 8; ++q)
          *reinterpret_cast<uint4 *>(base + 128 + q * 16) = NX == 2 ? sl[q] : make_uint4(0u, 0u, 0u, 0u);
      }
      gt_fence_async_smem();
      __syncwarp();
      if (lane == 0) gt_arrive(&S.bar[GB_BFULL + b]);
      return true;
    };
    bool eok = true;
    if (my > 0) eok = stage_uw(0);
    if (my > 1 && eok) eok = stage_uw(1);
    const int jl = e >> 3, p = e & 7;
    for (int i = 0; i < my && eok; ++i) {
      const int b = i & 1;
      const int c = blockIdx.x + i * gridDim.x;
      if (!gt_wait(&S.bar[GB_CDONE + b], (uint32_t)((i >> 1) & 1), abort)) break;
      t5_fence_after();
      const int eu = b ? eu1 : eu0, ew = b ? ew1 : ew0;
      for (int mb = 0; mb < NMB; ++mb) {
        float v[16];
        t5_ld16(tbase + ((uint32_t)(32 * warp) << 16) + (uint32_t)(b * NMB * 16 + mb * 16), v);
        const int j = mb * 16 + jl;
        const int ej = (j < J) ? gt_vscale(g, j, c * ct, min(ct, ntiles - c * ct)) : -128;
#pragma unroll
        for (int x = 0; x < NX; ++x) {
          // Y_k = sum_q D_kq 2^(7(7-q)) = H 2^42 + R, then weight 2^(8(6-k)) of byte k (slot 7 holds zeros)
          const long long H =
              (long long)__float2int_rn(v[x * 8 + 0]) * 128 + (long long)__float2int_rn(v[x * 8 + 1]);
          long long R = 0;
#pragma unroll
          for (int q = 2; q < 8; ++q) R += (long long)__float2int_rn(v[x * 8 + q]) * (1ll << (7 * (7 - q)));
          long long hi;
          unsigned long long lo;
          gt_make128(H, R, p < 7 ? 8 * (6 - p) : 0, hi, lo);
#pragma unroll
          for (int off = 4; off > 0; off >>= 1) {
            const long long ohi = __shfl_xor_sync(0xffffffffu, hi, off);
            const unsigned long long olo = __shfl_xor_sync(0xffffffffu, lo, off);
            gt_add128(hi, lo, ohi, olo);
          }
          if (p == 0 && j < J && ej > -128) {
            const double val = gt_to_double(hi, lo) * gt_pow2(ej + (x ? ew : eu) - 111);
            gt_dd_add(S.pdd[(j * 2 + x) * 2], S.pdd[(j * 2 + x) * 2 + 1], val);
          }
        }
      }
      t5_fence_before();
      __syncwarp();
      if (lane == 0) gt_arrive(&S.bar[GB_TFREE + b]);
      if (i + 2 < my) eok = stage_uw(i + 2);
    }
  } else if (warp == GT_MWARP) {
    // ---------------- MMA issuer ----------------
    if (lane == 0) {
      int q = 0;
      bool ok = true;
      for (int i = 0; i < my && ok; ++i) {
        const int b = i & 1, u = i >> 1;
        if (!gt_wait(&S.bar[GB_BFULL + b], (uint32_t)(u & 1), abort)) { ok = false; break; }
        if (u >= 1 && !gt_wait(&S.bar[GB_TFREE + b], (uint32_t)((u - 1) & 1), abort)) { ok = false; break; }
        t5_fence_after();
        const uint32_t bbase = t5_smem(Bs + (size_t)b * GT_CTMAX * GT_BT);
        for (int t = 0; t < ct && ok; ++t)
          for (int mb = 0; mb < NMB; ++mb, ++q) {
            const int sa = q % GT_NA;
            if (!gt_wait(&S.bar[GB_AFULL + sa], (uint32_t)((q / GT_NA) & 1), abort)) { ok = false; break; }
            t5_fence_after();
            const uint32_t abase = t5_smem(As + (size_t)sa * GT_STAGE);
            const uint32_t dcol = tbase + (uint32_t)(b * NMB * 16 + mb * 16);
#pragma unroll
            for (int ks = 0; ks < 8; ++ks) {
              const uint64_t ad = t5_desc(abase + ks * 2 * GT_DLBO, GT_DLBO, 128);
              const uint64_t bd = t5_desc(bbase + (uint32_t)((t * 16 + 2 * ks) * GT_BLBO), GT_BLBO, 128);
              t5_mma(dcol, ad, bd, GT_IDESC, (t > 0 || ks > 0) ? 1u : 0u);
            }
            t5_commit(&S.bar[GB_AEMPTY + sa]);
          }
        if (ok) t5_commit(&S.bar[GB_CDONE + b]);
      }
      // every MMA issued has completed before TMEM is freed (bounded)
      t5_commit(&S.bar[GB_FIN]);
      if (!t5_wait(&S.bar[GB_FIN], 0)) *abort = 1;
    }
  } else {
    // ---------------- slicers: item = (column jl, 8-row group k8) of a 16-column stage, loads one stage ahead ----
    const int s = tid - 32 * GT_SW0;  // 0..255
    const int jl = s >> 4, k8 = s & 15;
    const int total = my * ct * NMB;
    int ovf = 0;
    // stage q -> (chunk c, tile t, column block mb), advanced without divisions: a cursor per look-ahead slot
    struct Cur {
      int mb, t, i;
    };
    auto step = [&](Cur &u) {
      if (++u.mb == NMB) {
        u.mb = 0;
        if (++u.t == ct) {
          u.t = 0;
          ++u.i;
        }
      }
    };
    auto where_c = [&](const Cur &u, int &c, int &t, int &j, long long &r0, bool &valid) {
      t = u.t;
      c = blockIdx.x + u.i * gridDim.x;
      j = u.mb * 16 + jl;
      r0 = ((long long)c * ct + t) * GT_R + 8 * k8;
      valid = j < J && c * ct + t < ntiles;
    };
    Cur cq = {0, 0, 0}, cn = {0, 0, 0};  // the stage being sliced, the next stage to load
    // the loads of the next two stages are in flight while a stage is sliced (about 32 KB per SM)
    double vn1[8], vn2[8];
    auto issue = [&](double *dst) {  // loads the stage at cursor cn, then advances it
      int c2, t2, j2;
      long long r2;
      bool v2;
      where_c(cn, c2, t2, j2, r2, v2);
      gt_load8(V + (size_t)j2 * a.ldv + r2, r2, n, v2, dst);
      step(cn);
    };
    if (total > 0) issue(vn1);
    if (total > 1) issue(vn2);
    for (int q = 0; q < total; ++q, step(cq)) {
      const int sa = q & (GT_NA - 1);
      int c, t, j;
      long long r0;
      bool valid;
      where_c(cq, c, t, j, r0, valid);
      double v[8];
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        v[k] = vn1[k];
        vn1[k] = vn2[k];
      }
      if (q + 2 < total) issue(vn2);
      const int ej = valid ? gt_vscale(g, j, c * ct, min(ct, ntiles - c * ct)) : 0;
      long long X[8];
#pragma unroll
      for (int k = 0; k < 8; ++k) X[k] = gt_fix55(v[k], ej, &ovf);
      uint4 sl[7];
      gt_bytes7(X, sl);
      if (q >= GT_NA && !gt_wait(&S.bar[GB_AEMPTY + sa], (uint32_t)(((q >> 2) - 1) & 1), abort)) break;
      unsigned char *dst = As + (size_t)sa * GT_STAGE + (size_t)k8 * GT_DLBO + (size_t)jl * 128;
#pragma unroll
      for (int k = 0; k < 7; ++k) *reinterpret_cast<uint4 *>(dst + k * 16) = sl[k];
      gt_fence_async_smem();
      __syncwarp();
      if (lane == 0) gt_arrive(&S.bar[GB_AFULL + sa]);
    }
    if (ovf) atomicExch(g.err, 2);
  }
  // ---------------- teardown, partials, merge ----------------
  t5_fence_before();
  __syncthreads();
  t5_fence_after();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tbase), "r"(GT_TMEM) : "memory");
  if (*abort && tid == 0) atomicExch(g.err, 1);
  // scalars: reduce the epilogue threads' sums (fixed order)
  if (warp < GT_EW) {
    for (int off = 16; off > 0; off >>= 1) {
      sc0 += __shfl_down_sync(0xffffffffu, sc0, off);
      sc1 += __shfl_down_sync(0xffffffffu, sc1, off);
      sc2 += __shfl_down_sync(0xffffffffu, sc2, off);
    }
    if (lane == 0) {
      S.red[8 + warp * 3] = sc0;
      S.red[9 + warp * 3] = sc1;
      S.red[10 + warp * 3] = sc2;
    }
  }
  __syncthreads();
  const int nsc = NX == 2 ? 3 : 1;
  double *pb = g.part + (size_t)blockIdx.x * g.pstride;  // [J * NX][hi, lo], then the scalars
  for (int o = tid; o < J * NX; o += GT_THREADS) {
    const int j = o / NX, x = o % NX;
    pb[2 * o] = S.pdd[(j * 2 + x) * 2];
    pb[2 * o + 1] = S.pdd[(j * 2 + x) * 2 + 1];
  }
  if (tid < nsc) {
    double v = 0.0;
    for (int w = 0; w < GT_EW; ++w) v += S.red[8 + w * 3 + tid];
    pb[2 * J * NX + tid] = v;
  }
  __threadfence();
  __syncthreads();
  if (tid == 0) s_last = (atomicAdd(&st->tickets[TK_DOT], 1u) == gridDim.x - 1);
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  for (int o = tid; o < J * NX + nsc; o += GT_THREADS) {
    if (o < J * NX) {
      double hi = 0.0, lo = 0.0;
      for (int b2 = 0; b2 < (int)gridDim.x; ++b2) {
        const double *q2 = g.part + (size_t)b2 * g.pstride + 2 * o;
        gt_dd_add(hi, lo, __ldcg(q2));
        gt_dd_add(hi, lo, __ldcg(q2 + 1));
      }
      res[o] = hi + lo;
    } else {
      double v = 0.0;
      for (int b2 = 0; b2 < (int)gridDim.x; ++b2) v += __ldcg(g.part + (size_t)b2 * g.pstride + 2 * J * NX + (o - J * NX));
      res[o] = v;
    }
  }
  __syncthreads();
  if (tid == 0) st->tickets[TK_DOT] = 0;
  gs_epilogue<NX>(a, res, mode);
}

// ---------------------------------------------------------------------------------------------------------------
// Half B
// ---------------------------------------------------------------------------------------------------------------
template <int NX>
__global__ void __maxnreg__(128) k_gs_update_tc(StepArgs a, int mode, GTArgs g) {
  KrylovState *st = a.st;
  if (st->stop) return;
  extern __shared__ __align__(1024) unsigned char sm[];
  __shared__ int s_last, s_es[2];
  const GTShared S = gt_shared(sm, GT_UPD_MISC);
  volatile int *abort = S.ints;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int n = a.n, J = a.J, NKS = (J + 15) / 16;
  const double sigma = st->sigma, invnu = st->invnu, tsig = st->tau_sigma;
  double *U = static_cast<double *>(a.U);
  double *W = static_cast<double *>(a.W);
  const double *V = static_cast<const double *>(a.V);
  const int ntiles = (n + GT_R - 1) / GT_R;
  const int my = blockIdx.x < ntiles ? (ntiles - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
  if (tid == 0) {
    for (int i = 0; i < 64; ++i) S.ints[i] = 0;
    s_es[0] = s_es[1] = 0;
    gt_init_barriers(S);
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(t5_smem(S.tslot)),
                 "r"(GT_TMEM)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  __syncthreads();
  unsigned char *As = sm + GT_AOFF;
  unsigned char *Bs = sm + GT_BOFF;
  // the scales of s and g (all threads), then their byte slices: [k8][x][8 slots (7 bytes, slot 7 zero)][8 columns]
  {
    int Es = 0, Eg = 0;
    for (int j = tid; j < J; j += GT_THREADS) {
      Es = max(Es, gt_expo(a.coef[j]));
      if (NX == 2) Eg = max(Eg, gt_expo(a.coef[J + j]));
    }
    for (int off = 16; off > 0; off >>= 1) {
      Es = max(Es, __shfl_xor_sync(0xffffffffu, Es, off));
      Eg = max(Eg, __shfl_xor_sync(0xffffffffu, Eg, off));
    }
    if (lane == 0) {
      atomicMax(&s_es[0], Es);
      atomicMax(&s_es[1], Eg);
    }
  }
  __syncthreads();
  const int es = gt_escale(s_es[0]), eg = gt_escale(s_es[1]);
  for (int it = tid; it < 2 * NKS * 2; it += GT_THREADS) {
    const int x = it & 1, k8 = it >> 1;  // coefficients j = 8 k8 .. 8 k8 + 7 of vector x
    long long X[8];
    int ovf = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      const int j = 8 * k8 + k;
      const double cv = (j < J && (x == 0 || NX == 2)) ? a.coef[x * J + j] : 0.0;
      X[k] = gt_fix55(cv, x ? eg : es, &ovf);
    }
    uint4 sl[7];
    gt_bytes7(X, sl);
    unsigned char *base = Bs + (size_t)(k8 * 2 + x) * 128;
#pragma unroll
    for (int q = 0; q < 7; ++q) *reinterpret_cast<uint4 *>(base + q * 16) = sl[q];
    *reinterpret_cast<uint4 *>(base + 7 * 16) = make_uint4(0u, 0u, 0u, 0u);
  }
  gt_fence_async_smem();
  t5_fence_before();
  __syncthreads();
  t5_fence_after();
  const uint32_t tbase = *S.tslot;
  double nrm = 0.0;

  if (warp < GT_EW) {
    // ---------------- epilogue warps: row e of each tile ----------------
    const int e = tid;
    for (int i = 0; i < my; ++i) {
      const int b = i & 1, slot = i & 3;
      const int T = blockIdx.x + i * gridDim.x;
      const long long r = (long long)T * GT_R + e;
      double u = 0.0, w = 0.0;
      if (r < n) {
        u = U[r];
        if (NX == 2) w = W[r];
      }
      // the tile's row scale: the largest recorded exponent of its columns (each warp on its own; the slicers
      // compute the same value)
      int etile = -128;
      for (int j = lane; j < J; j += 32) etile = max(etile, (int)g.vexp[(size_t)j * g.ldt + T]);
      for (int off = 16; off > 0; off >>= 1) etile = max(etile, __shfl_xor_sync(0xffffffffu, etile, off));
      if (!gt_wait(&S.bar[GB_CDONE + b], (uint32_t)((i >> 1) & 1), abort)) break;
      t5_fence_after();
      // per vector, the 13 levels k + q of the byte products, as exact 32-bit integer sums
      // (|D| <= 144 * 255^2 < 2^24, at most 7 products per level)
      double prod[2] = {0.0, 0.0};
#pragma unroll
      for (int x = 0; x < NX; ++x) {
        int lev[13];
#pragma unroll
        for (int L = 0; L < 13; ++L) lev[L] = 0;
#pragma unroll
        for (int k = 0; k < 7; ++k) {
          float v[16];
          t5_ld16(tbase + ((uint32_t)(32 * warp) << 16) + (uint32_t)(b * 128 + k * 16), v);
#pragma unroll
          for (int q = 0; q < 7; ++q) lev[k + q] += __float2int_rn(v[x * 8 + q]);
        }
        // X = sum_L lev_L 2^(8(12-L)) = A3 2^64 + B3 2^32 + C3, each part below 2^59 in magnitude
        long long A3 = 0, B3 = 0, C3 = 0;
#pragma unroll
        for (int L = 0; L < 13; ++L) {
          if (L < 5) A3 += (long long)lev[L] * (1ll << (8 * (4 - L)));
          else if (L < 9) B3 += (long long)lev[L] * (1ll << (8 * (8 - L)));
          else C3 += (long long)lev[L] * (1ll << (8 * (12 - L)));
        }
        const double xs = fma(__ll2double_rn(A3), 18446744073709551616.0,
                              fma(__ll2double_rn(B3), 4294967296.0, __ll2double_rn(C3)));
        // (V c)_r = 2^(etile + e_c - 110) X
        prod[x] = (etile > -128) ? xs * gt_pow2(etile + (x ? eg : es) - 110) : 0.0;
      }
      t5_fence_before();
      __syncwarp();
      if (lane == 0) gt_arrive(&S.bar[GB_TFREE + b]);
      int Eu = 0;
      if (r < n) {
        const double un = (sigma * u - prod[0]) * invnu;
        U[r] = un;
        Eu = gt_expo(un);
        if (NX == 2) {
          const double wo = w - prod[1] - tsig * u;
          W[r] = wo;
          nrm = fma(wo, wo, nrm);
        }
      }
      // the exponent of the new column v_j over this tile, read by later launches: the warps' maxima meet in a
      // per-tile slot; the last of the four warps to arrive writes the table entry
      for (int off = 16; off > 0; off >>= 1) Eu = max(Eu, __shfl_xor_sync(0xffffffffu, Eu, off));
      if (lane == 0) {
        S.ints[16 + 4 * slot + warp] = Eu;
        __threadfence_block();
        if (atomicAdd(&S.ints[12 + slot], 1) == GT_EW - 1) {
          int m = 0;
#pragma unroll
          for (int q = 0; q < GT_EW; ++q) m = max(m, *(volatile int *)&S.ints[16 + 4 * slot + q]);
          g.vexp[(size_t)a.j * g.ldt + T] = (signed char)gt_escale(m);
          S.ints[12 + slot] = 0;
        }
      }
    }
  } else if (warp == GT_MWARP) {
    if (lane == 0) {
      const uint32_t bbase = t5_smem(Bs);
      int q = 0;
      bool ok = true;
      for (int i = 0; i < my && ok; ++i) {
        const int b = i & 1, u = i >> 1;
        if (u >= 1 && !gt_wait(&S.bar[GB_TFREE + b], (uint32_t)((u - 1) & 1), abort)) { ok = false; break; }
        for (int ks = 0; ks < NKS; ++ks, ++q) {
          const int sa = q % GT_NA;
          if (!gt_wait(&S.bar[GB_AFULL + sa], (uint32_t)((q / GT_NA) & 1), abort)) { ok = false; break; }
          t5_fence_after();
          const uint32_t abase = t5_smem(As + (size_t)sa * GT_STAGE);
          const uint64_t bd = t5_desc(bbase + (uint32_t)(ks * 2 * 256), 256, 128);
#pragma unroll
          for (int k = 0; k < 7; ++k) {
            const uint64_t ad = t5_desc(abase + k * 4096, 2048, 128);
            t5_mma(tbase + (uint32_t)(b * 128 + k * 16), ad, bd, GT_IDESC, ks > 0 ? 1u : 0u);
          }
          t5_commit(&S.bar[GB_AEMPTY + sa]);
        }
        if (ok) t5_commit(&S.bar[GB_CDONE + b]);
      }
      t5_commit(&S.bar[GB_FIN]);
      if (!t5_wait(&S.bar[GB_FIN], 0)) *abort = 1;
    }
  } else {
    // ---------------- slicers: item = (row rl, 8-column group kg) of a 16-column stage, loads one stage ahead ----
    const int s = tid - 32 * GT_SW0;
    const int rl = s & 127, kg = s >> 7;
    const int total = my * NKS;
    int ovf = 0;
    // the loads of the next two stages are in flight while a stage is sliced
    double vn1[8], vn2[8];
    int lks = 0, li = 0;  // the next stage to load: column step lks of the tile li
    auto load = [&](double *v) {
      const int T = blockIdx.x + li * gridDim.x, ks = lks;
      if (++lks == NKS) {
        lks = 0;
        ++li;
      }
      const long long r = (long long)T * GT_R + rl;
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        const int j = ks * 16 + kg * 8 + k;
        v[k] = (j < J && r < n) ? __ldcs(V + (size_t)j * a.ldv + r) : 0.0;
      }
    };
    if (total > 0) load(vn1);
    if (total > 1) load(vn2);
    int etile = -128;
    int cks = 0, ci = 0;  // the stage being sliced
    for (int q = 0; q < total; ++q) {
      const int sa = q & (GT_NA - 1);
      const int T = blockIdx.x + ci * gridDim.x;
      if (cks == 0) {
        etile = -128;  // as the epilogue warps compute it
        for (int j = lane; j < J; j += 32) etile = max(etile, (int)g.vexp[(size_t)j * g.ldt + T]);
        for (int off = 16; off > 0; off >>= 1) etile = max(etile, __shfl_xor_sync(0xffffffffu, etile, off));
      }
      double v[8];
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        v[k] = vn1[k];
        vn1[k] = vn2[k];
      }
      if (q + 2 < total) load(vn2);
      if (++cks == NKS) {
        cks = 0;
        ++ci;
      }
      long long X[8];
#pragma unroll
      for (int k = 0; k < 8; ++k) X[k] = gt_fix55(v[k], etile, &ovf);
      uint4 sl[7];
      gt_bytes7(X, sl);
      if (q >= GT_NA && !gt_wait(&S.bar[GB_AEMPTY + sa], (uint32_t)(((q >> 2) - 1) & 1), abort)) break;
      unsigned char *dst = As + (size_t)sa * GT_STAGE + (size_t)((kg * 16 + (rl >> 3)) * 128 + (rl & 7) * 16);
#pragma unroll
      for (int k = 0; k < 7; ++k) *reinterpret_cast<uint4 *>(dst + k * 4096) = sl[k];
      gt_fence_async_smem();
      __syncwarp();
      if (lane == 0) gt_arrive(&S.bar[GB_AFULL + sa]);
    }
    if (ovf) atomicExch(g.err, 2);
  }
  t5_fence_before();
  __syncthreads();
  t5_fence_after();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tbase), "r"(GT_TMEM) : "memory");
  if (*abort && tid == 0) atomicExch(g.err, 1);
  if (NX == 1) return;
  // ||w'||^2: the epilogue threads' sums in a fixed order, per block, then the last block (as k_gs_update)
  if (warp < GT_EW) {
    for (int off = 16; off > 0; off >>= 1) nrm += __shfl_down_sync(0xffffffffu, nrm, off);
    if (lane == 0) S.red[warp] = nrm;
  }
  __syncthreads();
  double *pb = g.part;
  if (tid == 0) {
    double v = 0.0;
    for (int w = 0; w < GT_EW; ++w) v += S.red[w];
    pb[blockIdx.x] = v;
  }
  __threadfence();
  __syncthreads();
  if (tid == 0) s_last = (atomicAdd(&st->tickets[TK_UPD], 1u) == gridDim.x - 1);
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  if (tid == 0) {
    double v = 0.0;
    for (int b2 = 0; b2 < (int)gridDim.x; ++b2) v += __ldcg(pb + b2);
    const double beta = sqrt(v);
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

// the exponent of each 128-row tile of one basis column written by another kernel (one block per tile)
__global__ void k_record_vexp(const double *col, int n, signed char *vexp_col) {
  const long long r = (long long)blockIdx.x * GT_R + threadIdx.x;
  int E = r < n ? gt_expo(col[r]) : 0;
  for (int off = 16; off > 0; off >>= 1) E = max(E, __shfl_xor_sync(0xffffffffu, E, off));
  __shared__ int wm[GT_R / 32];
  if ((threadIdx.x & 31) == 0) wm[threadIdx.x >> 5] = E;
  __syncthreads();
  if (threadIdx.x == 0) {
    int m = 0;
    for (int w = 0; w < GT_R / 32; ++w) m = max(m, wm[w]);
    vexp_col[blockIdx.x] = (signed char)gt_escale(m);
  }
}

cudaError_t launch_record_vexp(const double *col, int n, signed char *vexp_col, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_record_vexp<<<(n + GT_R - 1) / GT_R, GT_R, 0, s>>>(col, n, vexp_col);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------------------------------------------
int gs_tc_max_columns() { return GT_MAXJ; }

// tiles per chunk of half A: the longest chunk that still leaves three chunks per block
static int gs_tc_chunk_tiles(int n, int grid) {
  const int ntiles = (n + GT_R - 1) / GT_R;
  for (int ct = GT_CTMAX; ct > 1; ct >>= 1)
    if ((ntiles + ct - 1) / ct >= 3 * grid) return ct;
  return 1;
}

size_t gs_tc_part_doubles() { return (size_t)num_sms() * (4 * GT_MAXJ + 8); }

cudaError_t launch_gs_dot_tc(const StepArgs &a, int nx, int mode, const GTArgs &g0, cudaStream_t s) {
  if (a.J < 1 || a.J > GT_MAXJ || nx < 1 || nx > 2) return cudaErrorInvalidValue;
  GTArgs g = g0;
  const int ntiles = (a.n + GT_R - 1) / GT_R;
  int grid = num_sms();
  g.ct = gs_tc_chunk_tiles(a.n, grid);
  const int nchunks = (ntiles + g.ct - 1) / g.ct;
  if (grid > nchunks) grid = nchunks;
  g.pstride = 4 * GT_MAXJ + 8;
  cudaError_t e;
  if (nx == 2) {
    e = cudaFuncSetAttribute(k_gs_dot_tc<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)GT_DOT_SMEM);
    if (e != cudaSuccess) return e;
    k_gs_dot_tc<2><<<grid, GT_THREADS, GT_DOT_SMEM, s>>>(a, mode, g);
  } else {
    e = cudaFuncSetAttribute(k_gs_dot_tc<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)GT_DOT_SMEM);
    if (e != cudaSuccess) return e;
    k_gs_dot_tc<1><<<grid, GT_THREADS, GT_DOT_SMEM, s>>>(a, mode, g);
  }
  return cudaGetLastError();
}

template <int NX>
static cudaError_t upd_go(const StepArgs &a, int mode, const GTArgs &g, int grid, cudaStream_t s) {
  const cudaError_t e =
      cudaFuncSetAttribute(k_gs_update_tc<NX>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)GT_UPD_SMEM);
  if (e != cudaSuccess) return e;
  k_gs_update_tc<NX><<<grid, GT_THREADS, GT_UPD_SMEM, s>>>(a, mode, g);
  return cudaGetLastError();
}

cudaError_t launch_gs_update_tc(const StepArgs &a, int nx, int mode, const GTArgs &g, cudaStream_t s) {
  if (a.J < 1 || a.J > GT_MAXJ || nx < 1 || nx > 2) return cudaErrorInvalidValue;
  const int ntiles = (a.n + GT_R - 1) / GT_R;
  int grid = num_sms();
  if (grid > ntiles) grid = ntiles;
  return nx == 2 ? upd_go<2>(a, mode, g, grid, s) : upd_go<1>(a, mode, g, grid, s);
}

}  // namespace ksg
