// k_gs_ix.cu -- the DCGS2 Gram-Schmidt pair for IEEE-double storage with every product exact on the integer pipes.
//
// GB300's FP64 pipe issues about 0.6 T FMA/s, so the FP64-FMA Gram-Schmidt kernels (two FMAs per 8-byte basis entry)
// stop near 2.4 TB/s, a third of the HBM rate.  The integer pipes carry no such bound: a 32 x 32 -> 64-bit
// multiply-add (IMAD.WIDE) is one instruction.  Here
//
//   a value v with |v| < 2^e becomes the 54-bit two's complement fixed point X = trunc(v 2^(53-e)) -- the whole
//   significand of every value in the top binade of its scale, fewer bits below it -- split as X = H 2^26 + L
//   (|H| < 2^27, |L| < 2^26, both with the sign of v) with integer operations only (ix_split53);
//   a product X_v X_u = HH 2^52 + (HL + LH) 2^26 + LL is four IMAD.WIDE, and the three partial sums of a run of
//   products stay exact in 64-bit integers (|HH| < 2^54, |HL|, |LL| < 2^53: runs of up to 256 products);
//   a run's sum is one exact 128-bit integer, then either rounded once to a double (half B, per row) or added to a
//   128-bit accumulator with a binary exponent (half A, per column: ix_acc_add drops bits 2^-106 below the scale).
//
// Scales.  The basis columns carry one exponent per column and 128-row tile (the int8 table that the update half, the
// tcgen05 restart and launch_record_vexp keep for every column they write).  Half A scales a column over a tile of
// 512 G rows by the largest exponent of its 4 G table entries, u and w by their largest exponent in the tile; half B
// scales a row of V by the largest exponent of its 128-row tile over the J columns, s and g by their largest
// exponent.  A value at or above its scale sets the error flag (the host reports PETSC_ERR_PLIB).
//
// Half A (dot): s = V^T u, b = V^T w.  A block takes tiles of 512 G rows (G = 1..4, picked for an even split over
// the grid).  Per tile, u and w (copied into shared memory one tile ahead by cp.async) are split against the tile's
// scales; then each warp takes one basis column at a time, its lanes over the rows (coalesced 16-byte loads, the next
// group of 16 rows per lane -- of this column, the next one or the next tile -- in flight while a group is consumed).
// A lane sums its 16 G rows of the column exactly in 64-bit integers; the 32 lanes' sums meet in a 128-bit butterfly
// and lane 0 adds the tile's exact column sum to the column's accumulator.  The block's columns are rounded once;
// the last block merges the block partials in block order (double-double) and runs the DCGS2 coefficient algebra
// (gs_epilogue).
//
// Half B (update): [v w'] = [(sigma u - V s) / nu, w - V g - tau sigma u].  Thread = two adjacent rows; per column one
// 16-byte load, the split of both entries and eight IMAD.WIDE per row; the next eight columns' loads in flight.  The
// FP64 update, ||w'||^2 and the recorded tile exponents of v follow.  Results are deterministic: fixed partitions,
// fixed orders, no floating-point atomics.
#include "common.cuh"
#include "gs_fixed.cuh"
#include "kernels.h"
#include "krylov_body.cuh"
#include "ks_types.h"

namespace ksg {

constexpr int IX_THREADS = 512;                 // half A: 16 warps, one basis column per warp at a time
constexpr int IX_WARPS = IX_THREADS / 32;
constexpr int IX_GROUP = 512;                   // rows per load group: lane l takes 2l + 64i, +1 (i < 8)
constexpr int IX_GMAX = 4;                      // groups per tile (the launcher picks 1..4 for balance)
constexpr int IX_TMAX = IX_GROUP * IX_GMAX;
constexpr int IX_MAXJ = 144;
constexpr int IU_THREADS = 256;                 // half B
constexpr int IU_ROWS = 2 * IU_THREADS;         // rows per pass of half B

// one product of split values into the three exact partial sums: four 32 x 32 -> 64-bit multiply-adds
KS_DEVICE void ix_madw(long long &acc, int a, int b) { asm("mad.wide.s32 %0, %1, %2, %0;" : "+l"(acc) : "r"(a), "r"(b)); }
KS_DEVICE void ix_mac(long long &hh, long long &mm, long long &ll, int Hv, int Lv, int Hx, int Lx) {
  ix_madw(hh, Hv, Hx);
  ix_madw(mm, Hv, Lx);
  ix_madw(mm, Lv, Hx);
  ix_madw(ll, Lv, Lx);
}

// ---------------------------------------------------------------------------------------------------------------
// Half A
// ---------------------------------------------------------------------------------------------------------------
// 16-byte asynchronous global -> shared copy of `bytes` (0, 8 or 16) valid bytes, the rest zero-filled
KS_DEVICE void ix_cp16(void *dst, const void *src, int bytes) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"((uint32_t)__cvta_generic_to_shared(dst)),
               "l"(src), "r"(bytes)
               : "memory");
}
KS_DEVICE void ix_cp_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
KS_DEVICE void ix_cp_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// dynamic shared memory of half A: raw u, w of two tiles (copied one tile ahead), the split pairs of one tile, the
// per-column accumulators
constexpr size_t IXD_RAW = 0;                                           // double [2][2][IX_TMAX]
constexpr size_t IXD_SU = IXD_RAW + 2 * 2 * IX_TMAX * sizeof(double);   // int2 [u, w][IX_TMAX]
constexpr size_t IXD_ACC = IXD_SU + 2 * IX_TMAX * sizeof(int2);         // IxAcc [IX_MAXJ][2]
constexpr size_t IXD_SMEM = IXD_ACC + IX_MAXJ * 2 * sizeof(IxAcc);

template <int NX>
__global__ void __launch_bounds__(IX_THREADS, 1) k_gs_dot_ix(StepArgs a, int mode, GTArgs g) {
  KrylovState *st = a.st;
  if (st->stop) return;
  extern __shared__ __align__(16) unsigned char smx[];
  double *raw = reinterpret_cast<double *>(smx + IXD_RAW);  // [buffer][u, w][row]
  int2 *su = reinterpret_cast<int2 *>(smx + IXD_SU);        // (H, L) of u, then of w, per row of the tile
  IxAcc *cacc = reinterpret_cast<IxAcc *>(smx + IXD_ACC);   // [column][vector]
  __shared__ int emx[IX_THREADS / 32][2];
  __shared__ double sred[IX_THREADS / 32][3];
  __shared__ double res[IX_MAXJ * 2 + 4];
  __shared__ int s_last;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int n = a.n, J = a.J;
  const int G = g.ct, TR = IX_GROUP * G;                   // groups per tile, rows per tile
  const int ntile = (n + TR - 1) / TR, ntiles128 = (n + 127) >> 7;
  const int nk = warp < J ? (J - warp + IX_WARPS - 1) / IX_WARPS : 0;  // columns of this warp: warp + 16 kk
  const double sigma = st->sigma;
  const double *U = static_cast<const double *>(a.U);
  const double *W = static_cast<const double *>(a.W);
  const double *V = static_cast<const double *>(a.V);
  int flag = 0;
  double sc0 = 0.0, sc1 = 0.0, sc2 = 0.0;  // u.u, u.w, w.w of the staged rows
  for (int i = tid; i < J * NX; i += IX_THREADS) ix_acc_zero(cacc[i]);

  // raw u, w rows of tile t into buffer b: pairs of rows (2p, 2p + 1), zero-filled past n
  auto copy_raw = [&](int t, int b) {
    if (t >= ntile) return;
    const long long r0 = (long long)t * TR;
    for (int p = tid; 2 * p < TR; p += IX_THREADS) {
      const long long r = r0 + 2 * p;
      const int bytes = r + 1 < n ? 16 : (r < n ? 8 : 0);
      const long long rs = bytes ? r : 0;
      ix_cp16(raw + (size_t)(2 * b) * IX_TMAX + 2 * p, U + rs, bytes);
      if (NX == 2) ix_cp16(raw + (size_t)(2 * b + 1) * IX_TMAX + 2 * p, W + rs, bytes);
    }
    ix_cp_commit();
  };
  // one load group of a column: rows t TR + 512 gq + 2 lane + 64 i (+1), i < 8
  auto load_item = [&](int t, int kk, int gq, double (&v)[16]) {
    const double *col = V + (size_t)(warp + IX_WARPS * kk) * a.ldv;
    const long long rb = (long long)t * TR + IX_GROUP * gq + 2 * lane;
    if (rb + 64 * 7 + 1 < n) {
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        const double2 x = __ldcs(reinterpret_cast<const double2 *>(col + rb + 64 * i));
        v[2 * i] = x.x;
        v[2 * i + 1] = x.y;
      }
    } else {
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        const long long r = rb + 64 * i;
        v[2 * i] = r < n ? col[r] : 0.0;
        v[2 * i + 1] = r + 1 < n ? col[r + 1] : 0.0;
      }
    }
  };

  int t = blockIdx.x;
  copy_raw(t, 0);
  // the software pipeline alternates between two load buffers (par: the one holding the current group)
  double bA[16], bB[16];
  int par = 0;
  if (nk > 0 && t < ntile) load_item(t, 0, 0, bA);
  for (int it = 0; t < ntile; ++it, t += gridDim.x) {
    const int b = it & 1;
    // ---- stage the tile's u, w as split pairs against the tile's scales ----
    ix_cp_wait_all();
    __syncthreads();  // raw[b] complete; every warp is done with the previous tile's pairs
    copy_raw(t + (int)gridDim.x, b ^ 1);
    const double *ru = raw + (size_t)(2 * b) * IX_TMAX, *rw = raw + (size_t)(2 * b + 1) * IX_TMAX;
    int Eu = 0, Ew = 0;
    for (int r = tid; r < TR; r += IX_THREADS) {
      const double u = ru[r] * sigma;
      sc0 = fma(u, u, sc0);
      Eu = max(Eu, gt_expo(u));
      if (NX == 2) {
        const double w = rw[r];
        sc1 = fma(u, w, sc1);
        sc2 = fma(w, w, sc2);
        Ew = max(Ew, gt_expo(w));
      }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      Eu = max(Eu, __shfl_xor_sync(0xffffffffu, Eu, off));
      Ew = max(Ew, __shfl_xor_sync(0xffffffffu, Ew, off));
    }
    if (lane == 0) {
      emx[warp][0] = Eu;
      emx[warp][1] = Ew;
    }
    __syncthreads();
    Eu = 0;
    Ew = 0;
#pragma unroll
    for (int q = 0; q < IX_WARPS; ++q) {
      Eu = max(Eu, emx[q][0]);
      Ew = max(Ew, emx[q][1]);
    }
    const int eu = gt_escale(Eu), ew = gt_escale(Ew);
    for (int r = tid; r < TR; r += IX_THREADS) {
      int Hu, Lu, Hw = 0, Lw = 0;
      ix_split53(ru[r] * sigma, eu, Hu, Lu, flag);
      if (NX == 2) ix_split53(rw[r], ew, Hw, Lw, flag);
      su[r] = make_int2(Hu, Lu);
      su[IX_TMAX + r] = make_int2(Hw, Lw);
    }
    __syncthreads();  // pairs visible; emx free for the next tile
    // ---- the warp's columns: lanes over rows, one column at a time ----
    const int t128 = (int)(((long long)t * TR) >> 7);
    const int nt128 = min(TR >> 7, ntiles128 - t128);
    for (int kk = 0; kk < nk; ++kk) {
      const int c = warp + IX_WARPS * kk;
      int ec = lane < nt128 ? (int)g.vexp[(size_t)c * g.ldt + t128 + lane] : -128;
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) ec = max(ec, __shfl_xor_sync(0xffffffffu, ec, off));
      long long hh[NX], mm[NX], ll[NX];
#pragma unroll
      for (int x = 0; x < NX; ++x) {
        hh[x] = 0;
        mm[x] = 0;
        ll[x] = 0;
      }
      // one group: the next one is loaded (of this column, the next column, or this warp's first column in the next
      // tile) while this one is consumed
      auto group = [&](int gq, const double (&cv)[16], double (&nv)[16]) {
        if (gq + 1 < G) load_item(t, kk, gq + 1, nv);
        else if (kk + 1 < nk) load_item(t, kk + 1, 0, nv);
        else if (t + (int)gridDim.x < ntile) load_item(t + (int)gridDim.x, 0, 0, nv);
        const int rb = IX_GROUP * gq + 2 * lane;
#pragma unroll
        for (int i = 0; i < 8; ++i) {
          const int4 pu = *reinterpret_cast<const int4 *>(su + rb + 64 * i);
          const int4 pw = NX == 2 ? *reinterpret_cast<const int4 *>(su + IX_TMAX + rb + 64 * i) : make_int4(0, 0, 0, 0);
          int Hv, Lv;
          ix_split53(cv[2 * i], ec, Hv, Lv, flag);
          ix_mac(hh[0], mm[0], ll[0], Hv, Lv, pu.x, pu.y);
          if (NX == 2) ix_mac(hh[NX - 1], mm[NX - 1], ll[NX - 1], Hv, Lv, pw.x, pw.y);
          ix_split53(cv[2 * i + 1], ec, Hv, Lv, flag);
          ix_mac(hh[0], mm[0], ll[0], Hv, Lv, pu.z, pu.w);
          if (NX == 2) ix_mac(hh[NX - 1], mm[NX - 1], ll[NX - 1], Hv, Lv, pw.z, pw.w);
        }
      };
      for (int gq = 0; gq < G; ++gq) {
        if (par == 0) group(gq, bA, bB);
        else group(gq, bB, bA);
        par ^= 1;
      }
      // the column's exact sum over the tile: 128-bit butterfly over the lanes, folded by lane 0
#pragma unroll
      for (int x = 0; x < NX; ++x) {
        long long phi;
        unsigned long long plo;
        ix_combine(hh[x], mm[x], ll[x], phi, plo);
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
          const long long ohi = __shfl_xor_sync(0xffffffffu, phi, off);
          const unsigned long long olo = __shfl_xor_sync(0xffffffffu, plo, off);
          gt_add128(phi, plo, ohi, olo);
        }
        if (lane == 0 && ec > -128) ix_acc_add(cacc[c * NX + x], phi, plo, ec + (x ? ew : eu) - 106);
      }
    }
  }
  ix_cp_wait_all();
  if (flag < 0) atomicExch(g.err, 2);
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    sc0 += __shfl_down_sync(0xffffffffu, sc0, off);
    sc1 += __shfl_down_sync(0xffffffffu, sc1, off);
    sc2 += __shfl_down_sync(0xffffffffu, sc2, off);
  }
  if (lane == 0) {
    sred[warp][0] = sc0;
    sred[warp][1] = sc1;
    sred[warp][2] = sc2;
  }
  __syncthreads();
  // ---- per-block partials: the columns' sums (rounded once; [hi, lo] with lo = 0), then the scalars ----
  const int nsc = NX == 2 ? 3 : 1;
  double *pb = g.part + (size_t)blockIdx.x * g.pstride;
  for (int o = tid; o < J * NX; o += IX_THREADS) {
    const IxAcc A = cacc[o];
    pb[2 * o] = A.k == INT_MIN ? 0.0 : ix_to_double(A.hi, A.lo, A.k);
    pb[2 * o + 1] = 0.0;
  }
  if (tid < nsc) {
    double v = 0.0;
    for (int q = 0; q < IX_WARPS; ++q) v += sred[q][tid];
    pb[2 * J * NX + tid] = v;
  }
  __threadfence();
  __syncthreads();
  if (tid == 0) s_last = (atomicAdd(&st->tickets[TK_DOT], 1u) == gridDim.x - 1);
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  for (int o = tid; o < J * NX + nsc; o += IX_THREADS) {
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

// ||w'||^2 of half B: the threads' sums in a fixed order, per block, then the last block turns it into the next
// step's scale (or a breakdown)
KS_DEVICE void ix_update_norm(const StepArgs &a, double *pb, double nrm) {
  KrylovState *st = a.st;
  __shared__ double sred[IU_THREADS / 32];
  __shared__ int s_last;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) nrm += __shfl_down_sync(0xffffffffu, nrm, off);
  if (lane == 0) sred[warp] = nrm;
  __syncthreads();
  if (tid == 0) {
    double v = 0.0;
    for (int q = 0; q < IU_THREADS / 32; ++q) v += sred[q];
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

// ---------------------------------------------------------------------------------------------------------------
// Half B
// ---------------------------------------------------------------------------------------------------------------
template <int NX>
__global__ void __launch_bounds__(IU_THREADS, 2) k_gs_update_ix(StepArgs a, int mode, GTArgs g) {
  KrylovState *st = a.st;
  if (st->stop) return;
  __shared__ int4 cp[IX_MAXJ];                 // (H_s, L_s, H_g, L_g) per column
  __shared__ int s_es[2];
  __shared__ int s_tm[2][IU_ROWS / 128];       // per pass (two in turn), per 128-row tile: the exponent of v_j
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int n = a.n, J = a.J;
  const double sigma = st->sigma, invnu = st->invnu, tsig = st->tau_sigma;
  double *U = static_cast<double *>(a.U);
  double *W = static_cast<double *>(a.W);
  const double *V = static_cast<const double *>(a.V);
  const int ntiles = (n + 127) >> 7;
  const int npass = (n + IU_ROWS - 1) / IU_ROWS;
  const bool record = mode != GS_COMBINE;
  if (tid < 2) s_es[tid] = 0;
  if (tid < 2 * (IU_ROWS / 128)) s_tm[tid / (IU_ROWS / 128)][tid % (IU_ROWS / 128)] = 0;
  __syncthreads();
  {
    int Es = 0, Eg = 0;
    for (int j = tid; j < J; j += IU_THREADS) {
      Es = max(Es, gt_expo(a.coef[j]));
      if (NX == 2) Eg = max(Eg, gt_expo(a.coef[J + j]));
    }
#pragma unroll
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
  int flag = 0;
  for (int j = tid; j < J; j += IU_THREADS) {
    int hs, ls, hg = 0, lg = 0;
    ix_split53(a.coef[j], es, hs, ls, flag);
    if (NX == 2) ix_split53(a.coef[J + j], eg, hg, lg, flag);
    cp[j] = make_int4(hs, ls, hg, lg);
  }
  __syncthreads();
  double nrm = 0.0;
  for (int p = blockIdx.x, i = 0; p < npass; p += gridDim.x, ++i) {
    const long long r = (long long)p * IU_ROWS + 2 * tid;
    const int T = (int)(((long long)p * IU_ROWS + 64 * warp) >> 7);  // the 128-row tile of this warp's 64 rows
    // the rows' scale: the largest recorded exponent of the tile over the J columns
    int et = -128;
    if (T < ntiles)
      for (int c = lane; c < J; c += 32) et = max(et, (int)g.vexp[(size_t)c * g.ldt + T]);
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) et = max(et, __shfl_xor_sync(0xffffffffu, et, off));
    const bool two = r + 1 < n, one = r < n;
    long long hh[2][NX], mm[2][NX], ll[2][NX];
#pragma unroll
    for (int e = 0; e < 2; ++e)
#pragma unroll
      for (int x = 0; x < NX; ++x) {
        hh[e][x] = 0;
        mm[e][x] = 0;
        ll[e][x] = 0;
      }
    if (one && et > -128) {
      const double *colp = V + r;
      // groups of 8 columns in two buffers: the next group's loads in flight while the current one is consumed
      auto loadg = [&](int c0, double (&x0)[8], double (&x1)[8]) {
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          if (c0 + q < J) {
            if (two) {
              const double2 v = __ldcs(reinterpret_cast<const double2 *>(colp + (size_t)(c0 + q) * a.ldv));
              x0[q] = v.x;
              x1[q] = v.y;
            } else {
              x0[q] = colp[(size_t)(c0 + q) * a.ldv];
              x1[q] = 0.0;
            }
          }
        }
      };
      auto consume = [&](int c0, const double (&x0)[8], const double (&x1)[8]) {
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          if (c0 + q < J) {
            const int4 cq = cp[c0 + q];
            int H0, L0, H1, L1;
            ix_split53(x0[q], et, H0, L0, flag);
            ix_split53(x1[q], et, H1, L1, flag);
            ix_mac(hh[0][0], mm[0][0], ll[0][0], H0, L0, cq.x, cq.y);
            ix_mac(hh[1][0], mm[1][0], ll[1][0], H1, L1, cq.x, cq.y);
            if (NX == 2) {
              ix_mac(hh[0][NX - 1], mm[0][NX - 1], ll[0][NX - 1], H0, L0, cq.z, cq.w);
              ix_mac(hh[1][NX - 1], mm[1][NX - 1], ll[1][NX - 1], H1, L1, cq.z, cq.w);
            }
          }
        }
      };
      double a0[8], a1[8], b0[8], b1[8];
      loadg(0, a0, a1);
      for (int c0 = 0; c0 < J; c0 += 16) {
        if (c0 + 8 < J) loadg(c0 + 8, b0, b1);
        consume(c0, a0, a1);
        if (c0 + 8 >= J) break;
        if (c0 + 16 < J) loadg(c0 + 16, a0, a1);
        consume(c0 + 8, b0, b1);
      }
    }
    int Ev = 0;
    if (one) {
      // (V c)_r = 2^(et + e_c - 106) P, rounded once
      double prod[2][NX];
#pragma unroll
      for (int e = 0; e < 2; ++e)
#pragma unroll
        for (int x = 0; x < NX; ++x) {
          long long phi;
          unsigned long long plo;
          ix_combine(hh[e][x], mm[e][x], ll[e][x], phi, plo);
          prod[e][x] = et > -128 ? ix_to_double(phi, plo, et + (x ? eg : es) - 106) : 0.0;
        }
      double u0, u1 = 0.0, w0 = 0.0, w1 = 0.0;
      if (two) {
        const double2 uu = *reinterpret_cast<const double2 *>(U + r);
        u0 = uu.x;
        u1 = uu.y;
        if (NX == 2) {
          const double2 ww = *reinterpret_cast<const double2 *>(W + r);
          w0 = ww.x;
          w1 = ww.y;
        }
      } else {
        u0 = U[r];
        if (NX == 2) w0 = W[r];
      }
      const double v0 = (sigma * u0 - prod[0][0]) * invnu, v1 = (sigma * u1 - prod[1][0]) * invnu;
      Ev = max(gt_expo(v0), two ? gt_expo(v1) : 0);
      if (two) *reinterpret_cast<double2 *>(U + r) = make_double2(v0, v1);
      else U[r] = v0;
      if (NX == 2) {
        const double o0 = w0 - prod[0][NX - 1] - tsig * u0, o1 = w1 - prod[1][NX - 1] - tsig * u1;
        if (two) *reinterpret_cast<double2 *>(W + r) = make_double2(o0, o1);
        else W[r] = o0;
        nrm = fma(o0, o0, nrm);
        if (two) nrm = fma(o1, o1, nrm);
      }
    }
    // the exponents of the new column over this pass's tiles, read by later launches
    if (record) {
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) Ev = max(Ev, __shfl_xor_sync(0xffffffffu, Ev, off));
      if (lane == 0) atomicMax(&s_tm[i & 1][warp >> 1], Ev);
      __syncthreads();
      if (tid < IU_ROWS / 128) {
        const int Tt = p * (IU_ROWS / 128) + tid;
        if (Tt < ntiles) g.vexp[(size_t)a.j * g.ldt + Tt] = (signed char)gt_escale(s_tm[i & 1][tid]);
        s_tm[i & 1][tid] = 0;
      }
    }
  }
  if (flag < 0) atomicExch(g.err, 2);
  if constexpr (NX == 2) ix_update_norm(a, g.part, nrm);
}

// ---------------------------------------------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------------------------------------------
int gs_ix_max_columns() { return IX_MAXJ; }

// groups per tile of half A: the largest G in 4..1 whose tiles spread over the grid within 2% of an even split
// (fewer lane reductions per column), else the most even one
static int gs_ix_groups(int n, int sms) {
  int best = 1;
  double best_w = 1e30;
  for (int G = IX_GMAX; G >= 1; --G) {
    const long long nt = ((long long)n + IX_GROUP * G - 1) / (IX_GROUP * G);
    const long long gr = nt < sms ? nt : sms;
    const double w = (double)((nt + gr - 1) / gr * gr) / (double)nt;
    if (w <= 1.02) return G;
    if (w < best_w) {
      best_w = w;
      best = G;
    }
  }
  return best;
}

cudaError_t launch_gs_dot_ix(const StepArgs &a, int nx, int mode, const GTArgs &g0, cudaStream_t s) {
  if (a.J < 1 || a.J > IX_MAXJ || nx < 1 || nx > 2) return cudaErrorInvalidValue;
  GTArgs g = g0;
  g.ct = gs_ix_groups(a.n, num_sms());
  const int ntile = (int)(((long long)a.n + IX_GROUP * g.ct - 1) / (IX_GROUP * g.ct));
  int grid = num_sms();
  if (grid > ntile) grid = ntile;
  g.pstride = 4 * IX_MAXJ + 8;
  if ((size_t)grid * g.pstride > gs_tc_part_doubles()) return cudaErrorInvalidValue;
  cudaError_t e;
  if (nx == 2) {
    e = cudaFuncSetAttribute(k_gs_dot_ix<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)IXD_SMEM);
    if (e != cudaSuccess) return e;
    k_gs_dot_ix<2><<<grid, IX_THREADS, IXD_SMEM, s>>>(a, mode, g);
  } else {
    e = cudaFuncSetAttribute(k_gs_dot_ix<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)IXD_SMEM);
    if (e != cudaSuccess) return e;
    k_gs_dot_ix<1><<<grid, IX_THREADS, IXD_SMEM, s>>>(a, mode, g);
  }
  return cudaGetLastError();
}

cudaError_t launch_gs_update_ix(const StepArgs &a, int nx, int mode, const GTArgs &g, cudaStream_t s) {
  if (a.J < 1 || a.J > IX_MAXJ || nx < 1 || nx > 2) return cudaErrorInvalidValue;
  const int npass = (a.n + IU_ROWS - 1) / IU_ROWS;
  int grid = 2 * num_sms();
  if (grid > npass) grid = npass;
  if ((size_t)grid > gs_tc_part_doubles()) return cudaErrorInvalidValue;
  if (nx == 2) k_gs_update_ix<2><<<grid, IU_THREADS, 0, s>>>(a, mode, g);
  else k_gs_update_ix<1><<<grid, IU_THREADS, 0, s>>>(a, mode, g);
  return cudaGetLastError();
}

}  // namespace ksg
