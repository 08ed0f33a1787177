// k_ds_hep.cu -- projected problem of the symmetric Krylov-Schur iteration, solved on the device in FP64.
//
// One thread block per projected problem.  Follows DSSolve_HEP_QR (src/sys/classes/ds/impls/hep/dshep.c:383-426):
// the arrowhead block left by the previous restart is reduced to tridiagonal form by Givens rotations chased to
// the top-left corner (DSArrowTridiag, dshep.c:221-262), then the tridiagonal problem is solved by implicit QL
// with Wilkinson shifts (the algorithm LAPACK's steqr implements), the eigenvalues are sorted ascending and then
// by the requested criterion (DSSort_HEP, dshep.c:323-347 with dspriv.c:226-245), the extra row
// b = beta * Q(n-1, :) is formed (DSUpdateExtraRow_HEP, dshep.c:349-381), and the convergence test, stopping
// test and restart sizes of EPSSolve_KrylovSchur_Default (krylovschur.c:270-322, epskrylov.c:207-295,
// epsdefault.c:224-232,290-302) are evaluated so the host reads only a small control record.
//
// The rotation sequences are computed by one thread and applied to the rows of Q by all threads; Q lives in
// shared memory for n <= 144, and in place in the caller's Q (global memory, L2-resident) up to n = 1024.
#include <float.h>

#include "batch_types.h"
#include "common.cuh"
#include "kernels.h"
#include "ks_types.h"

namespace ksg {

constexpr int DS_THREADS = 256;
constexpr int DS_MAXN = 144;
constexpr int DS_WIDE_MAXN = 1024;

// per-index scratch of one projected solve: shared arrays for n <= 144, carved from dynamic shared memory above
struct DSHepMem {
  double *sd, *se, *rc, *rs, *serr, *dtmp, *rc2, *rs2;  // rc2, rs2: the second buffer of QL sweep rotations
  int *sperm, *sw_a, *sw_b, *perm2, *comp, *where, *at;
  double *Qs;  // n x n, column-major with leading dimension ldq
  int ldq;
  int inplace;  // Qs is a.Q itself (ldq = a.ld): no copy in or out
};

static inline size_t ds_wide_smem(int n) { return (size_t)n * (8 * sizeof(double) + 7 * sizeof(int)); }

KS_DEVICE DSHepMem ds_wide_mem(unsigned char *raw, int n, double *Q, int ld) {
  DSHepMem m;
  double *dp = reinterpret_cast<double *>(raw);
  m.sd = dp; m.se = dp + n; m.rc = dp + 2 * n; m.rs = dp + 3 * n; m.serr = dp + 4 * n; m.dtmp = dp + 5 * n;
  m.rc2 = dp + 6 * n; m.rs2 = dp + 7 * n;
  int *ip = reinterpret_cast<int *>(dp + 8 * n);
  m.sperm = ip; m.sw_a = ip + n; m.sw_b = ip + 2 * n; m.perm2 = ip + 3 * n; m.comp = ip + 4 * n;
  m.where = ip + 5 * n; m.at = ip + 6 * n;
  m.Qs = Q;
  m.ldq = ld;
  m.inplace = 1;
  return m;
}

KS_DEVICE void ds_givens(double f, double g, double &c, double &s, double &r) {
  if (g == 0.0) {
    c = 1.0; s = 0.0; r = f;
  } else if (f == 0.0) {
    c = 0.0; s = copysign(1.0, g); r = fabs(g);
  } else {
    // d = hypot(f, g) by one reciprocal square root (a dependent FP64 square root and division cost about 690 and
    // 440 cycles on GB300); hypot where the sum of squares could underflow
    const double t2 = fma(f, f, g * g);
    if (t2 < 1e-280) {
      const double d = hypot(f, g);
      c = fabs(f) / d;
      r = copysign(d, f);
      s = g / r;
    } else {
      const double di = rsqrt(t2);
      c = fabs(f) * di;
      r = copysign(t2 * di, f);
      s = (f < 0.0 ? -g : g) * di;  // g / r, r carrying the sign of f
    }
  }
}

// criterion comparison (slepcsc.c:152-267): -1 if a goes first, 1 if b goes first, 0 if tied; 7 and 8 measure
// the distance to the target
KS_DEVICE int ds_compare(int which, double target, double ar, double ai, double br, double bi) {
  double a, b;
  switch (which) {
    case 7: a = hypot(ar - target, ai); b = hypot(br - target, bi); return a > b ? 1 : (a < b ? -1 : 0);
    case 8: a = fabs(ar - target); b = fabs(br - target); return a > b ? 1 : (a < b ? -1 : 0);
    case 1: a = hypot(ar, ai); b = hypot(br, bi); return a < b ? 1 : (a > b ? -1 : 0);
    case 2: a = hypot(ar, ai); b = hypot(br, bi); return a > b ? 1 : (a < b ? -1 : 0);
    case 3: return ar < br ? 1 : (ar > br ? -1 : 0);
    case 4: return ar > br ? 1 : (ar < br ? -1 : 0);
    case 5: a = fabs(ai); b = fabs(bi); return a < b ? 1 : (a > b ? -1 : 0);
    case 6: a = fabs(ai); b = fabs(bi); return a > b ? 1 : (a < b ? -1 : 0);
    default: return 0;
  }
}

// the small solver's scratch: shared arrays, Q in dynamic shared memory with leading dimension n
#define DS_SMALL_MEM(m, Qshared, nn)                                                                          \
  __shared__ double sd_[DS_MAXN], se_[DS_MAXN], rc_[DS_MAXN], rs_[DS_MAXN], serr_[DS_MAXN], dtmp_[DS_MAXN],  \
      rc2_[DS_MAXN], rs2_[DS_MAXN];                                                                          \
  __shared__ int sperm_[DS_MAXN], swa_[DS_MAXN], swb_[DS_MAXN], perm2_[DS_MAXN], comp_[DS_MAXN],              \
      where_[DS_MAXN], at_[DS_MAXN];                                                                         \
  DSHepMem m = {sd_,    se_,    rc_,   rs_,    serr_,  dtmp_, rc2_,    rs2_, sperm_,                          \
                swa_,   swb_,   perm2_, comp_, where_, at_,   Qshared, nn,   0}

KS_DEVICE void ds_hep_body(const DSArgs &a, const DSHepMem &mem) {
  __shared__ int s_cmd2[2], s_lo2[2], s_hi2[2], s_nsw, s_fail;
  __shared__ double s_beta_e;
  double *sd = mem.sd, *se = mem.se, *rc = mem.rc, *rs = mem.rs, *serr = mem.serr;
  int *sperm = mem.sperm, *sw_a = mem.sw_a, *sw_b = mem.sw_b;
  double *Qs = mem.Qs;
  const int tid = threadIdx.x;
  const KrylovState *st = a.st;
  const int n = st ? st->m : a.n;  // actual size of the factorisation
  const size_t lq = mem.inplace ? (size_t)mem.ldq : (size_t)n;  // leading dimension of Qs
  const int flags = a.flags;
  const int l = a.l, k = a.k;
  const int nq = n;
  for (int i = tid; i < n; i += DS_THREADS) {
    sd[i] = a.d[i];
    se[i] = a.e[i];
  }
  if (flags & DS_DO_SOLVE) {
    for (int i = tid; i < n * n; i += DS_THREADS) Qs[(i % n) + (i / n) * lq] = ((i % n) == (i / n)) ? 1.0 : 0.0;
  } else if (!mem.inplace) {
    for (int i = tid; i < n * n; i += DS_THREADS) Qs[i] = a.Q[(i % n) + (size_t)(i / n) * a.ld];
  }
  if (tid == 0) s_fail = 0;
  __syncthreads();
  if (tid == 0) s_beta_e = se[n - 1];
  // ---- arrowhead -> tridiagonal on the block [l, k] ----
  const int n1 = ((flags & DS_DO_SOLVE) && a.raw && k - l + 1 > 0) ? k - l + 1 : 0;
  for (int j = 0; j < n1 - 2; ++j) {
    if (tid == 0) {
      double *d = sd + l, *e = se + l;
      double c, s, r;
      ds_givens(e[j + 1], e[j], c, s, r);
      e[j + 1] = r;
      s = -s;
      const double dj = d[j], dj1 = d[j + 1];
      e[j] = c * s * (dj1 - dj);
      d[j + 1] = s * s * dj + c * c * dj1;
      d[j] = c * c * dj + s * s * dj1;
      rc[0] = c;
      rs[0] = s;
      int t = 1;
      for (int i = j - 1; i >= 0; --i, ++t) {
        const double off = -s * e[i];
        e[i] = c * e[i];
        ds_givens(e[i + 1], off, c, s, r);
        e[i + 1] = r;
        s = -s;
        const double tt = (d[i] - d[i + 1]) * s - 2.0 * c * e[i];
        const double p = s * tt;
        d[i + 1] += p;
        d[i] -= p;
        e[i] = -e[i] - c * tt;
        rc[t] = c;
        rs[t] = s;
      }
    }
    __syncthreads();
    // rows 0..j+1 of the block; rotation t acts on block columns (j - t + 1 ... ) : t = 0 -> (j, j+1), t >= 1 -> (j-t, j-t+1)
    for (int r = tid; r < j + 2; r += DS_THREADS) {
      double *row = Qs + (l + r);
      for (int t = 0; t <= j; ++t) {
        const int p = (t == 0) ? j : j - t;
        const double c = rc[t], s = rs[t];
        double *x = row + (size_t)(l + p) * lq, *y = row + (size_t)(l + p + 1) * lq;
        const double xv = *x, yv = *y;
        *x = c * xv + s * yv;
        *y = c * yv - s * xv;
      }
    }
    __syncthreads();
  }
  // ---- implicit QL on [l, n) ----
  {
    // Thread 0 computes each sweep's rotations (the serial FP64 chain) into one of two buffers while the warps on
    // sub-partitions 1-3 apply the previous sweep's rotations to the rows of Q: the two overlap, and sub-partition
    // 0's FP64 pipe (thread 0's warp and warp 4) stays with the chain.
    int ll = 0, total = 0;  // thread 0 state (block-relative indices)
    const int m_blk = (flags & DS_DO_SOLVE) ? n - l : 0;
    double *d = sd + l, *e = se + l;
    double *rcb[2] = {rc, mem.rc2}, *rsb[2] = {rs, mem.rs2};
    if (tid == 0 && m_blk > 0) e[m_blk - 1] = 0.0;
    auto sweep = [&](int buf) {  // thread 0: the next sweep's rotations into buffer buf, or s_cmd2[buf] = 0
      double *rcw = rcb[buf], *rsw = rsb[buf];
      s_cmd2[buf] = 0;
      while (ll < m_blk) {
        int m;
        for (m = ll; m < m_blk - 1; ++m) {
          const double dd = fabs(d[m]) + fabs(d[m + 1]);
          if (fabs(e[m]) <= DBL_EPSILON * dd) break;
        }
        if (m == ll) { ++ll; continue; }
        if (++total > 30 * m_blk) { s_fail = 1; break; }
        double g = (d[ll + 1] - d[ll]) / (2.0 * e[ll]);
        double r = hypot(g, 1.0);
        g = d[m] - d[ll] + e[ll] / (g + copysign(r, g));
        double s = 1.0, c = 1.0, p = 0.0;
        int i;
        int under = 0;
        for (i = m - 1; i >= ll; --i) {
          const double f = s * e[i], b = c * e[i];
          // r = hypot(f, g), s = f / r, c = g / r by one reciprocal square root: on GB300 a dependent FP64
          // square root costs about 690 cycles and a division 440, and this recurrence is the solver's serial
          // chain (sums of squares far from overflow here: the operator is scaled into [2^-20, 2^20])
          const double t2 = fma(f, f, g * g);
          if (t2 < 1e-280) {
            r = hypot(f, g);
            e[i + 1] = r;
            if (r == 0.0) { d[i + 1] -= p; e[m] = 0.0; under = 1; break; }
            s = f / r;
            c = g / r;
          } else {
            const double ri = rsqrt(t2);
            r = t2 * ri;
            e[i + 1] = r;
            s = f * ri;
            c = g * ri;
          }
          g = d[i + 1] - p;
          r = (d[i] - g) * s + 2.0 * c * b;
          p = s * r;
          d[i + 1] = g + p;
          g = c * r - b;
          rcw[i] = c;
          rsw[i] = s;
        }
        if (!under) {
          d[ll] -= p;
          e[ll] = g;
          e[m] = 0.0;
        }
        s_lo2[buf] = under ? i + 1 : ll;
        s_hi2[buf] = m;  // rotations i = s_hi-1 down to s_lo
        s_cmd2[buf] = 1;
        break;
      }
    };
    if (tid == 0) sweep(0);
    __syncthreads();
    const int warp = tid >> 5, lane = tid & 31;
    const int aw = (warp & 3) ? (warp >> 2) * 3 + (warp & 3) - 1 : -1;  // warps 1-3, 5-7 -> 0..5
    constexpr int DS_APPLIERS = 6 * 32;
    for (int k = 0;; ++k) {
      const int cur = k & 1;
      if (s_cmd2[cur] == 0) break;
      if (tid == 0) {
        sweep(cur ^ 1);
      } else if (aw >= 0) {
        const int lo = s_lo2[cur], hi = s_hi2[cur];
        const double *rcr = rcb[cur], *rsr = rsb[cur];
        for (int r = aw * 32 + lane; r < nq; r += DS_APPLIERS) {
          double *row = Qs + r;
          // column l+i+1 of rotation i is column l+i of rotation i+1: carried in a register down the sweep
          double t = row[(size_t)(l + hi) * lq];
          for (int i = hi - 1; i >= lo; --i) {
            const double c = rcr[i], s = rsr[i];
            const double qi = row[(size_t)(l + i) * lq];
            row[(size_t)(l + i + 1) * lq] = s * qi + c * t;
            t = c * qi - s * t;
          }
          row[(size_t)(l + lo) * lq] = t;
        }
      }
      __syncthreads();
    }
    // the last off-diagonal slot holds the extra-row scalar beta, which steqr never touches
    if (tid == 0 && m_blk > 0) e[m_blk - 1] = s_beta_e;
  }
  // ---- ascending order (steqr) then sort by criterion (DSSort_HEP): one permutation, applied as swaps ----
  if (tid == 0) {
    const int m_blk = (flags & DS_DO_SOLVE) ? n - l : 0;
    for (int i = 0; i < n; ++i) sperm[i] = i;
    // ascending selection sort on the block
    for (int i = 0; i < m_blk - 1; ++i) {
      int kk = i;
      double p = sd[l + i];
      for (int j = i + 1; j < m_blk; ++j)
        if (sd[l + j] < p) { kk = j; p = sd[l + j]; }
      if (kk != i) {
        sd[l + kk] = sd[l + i];
        sd[l + i] = p;
        const int t = sperm[l + i]; sperm[l + i] = sperm[l + kk]; sperm[l + kk] = t;
      }
    }
    // insertion sort by criterion on indices (dspriv.c:226-245), over positions [l, n)
    int *perm2 = mem.perm2;
    for (int i = 0; i < n; ++i) perm2[i] = i;
    for (int i = l + 1; i < ((flags & DS_DO_SORT) ? n : 0); ++i) {
      const double re = sd[perm2[i]];
      int j = i - 1;
      int res = ds_compare(a.which, a.target, re, 0.0, sd[perm2[j]], 0.0);
      while (res < 0 && j >= l) {
        const int t = perm2[j]; perm2[j] = perm2[j + 1]; perm2[j + 1] = t;
        --j;
        if (j >= l) res = ds_compare(a.which, a.target, re, 0.0, sd[perm2[j]], 0.0);
      }
    }
    // composite: final column i = original column sperm[perm2[i]]
    double *dtmp = mem.dtmp;
    int *comp = mem.comp;
    for (int i = 0; i < n; ++i) { comp[i] = sperm[perm2[i]]; dtmp[i] = sd[perm2[i]]; }
    for (int i = 0; i < n; ++i) sd[i] = dtmp[i];
    // realise comp as a swap sequence on columns: position i must receive original column comp[i]
    int *where = mem.where, *at = mem.at;  // where[c]: current position of original column c; at[p]: column at p
    for (int i = 0; i < n; ++i) { where[i] = i; at[i] = i; }
    int nsw = 0;
    for (int i = 0; i < n; ++i) {
      const int c = comp[i];
      const int p = where[c];
      if (p != i) {
        sw_a[nsw] = i;
        sw_b[nsw] = p;
        ++nsw;
        const int ci = at[i];
        at[i] = c; where[c] = i;
        at[p] = ci; where[ci] = p;
      }
    }
    s_nsw = nsw;
  }
  __syncthreads();
  for (int r = tid; r < nq; r += DS_THREADS) {
    for (int t = 0; t < s_nsw; ++t) {
      double *x = Qs + r + (size_t)sw_a[t] * lq, *y = Qs + r + (size_t)sw_b[t] * lq;
      const double v = *x;
      *x = *y;
      *y = v;
    }
  }
  __syncthreads();
  // ---- extra row, convergence estimates ----
  const double beta = st ? st->beta_out : 0.0;
  const double beta_e = s_beta_e;
  for (int i = tid; i < n; i += DS_THREADS) {
    const double qlast = Qs[(n - 1) + (size_t)i * lq];
    if (flags & DS_DO_EXTRAROW) se[i] = beta_e * qlast;
    else if ((flags & DS_DO_SOLVE) && i < n - 1) se[i] = 0.0;
    const double w = fabs(sd[i]);
    serr[i] = ds_conv_errest(a, fabs(qlast) * beta, w);
  }
  __syncthreads();
  // ---- write back ----
  for (int i = tid; i < n; i += DS_THREADS) {
    a.d[i] = sd[i];
    a.e[i] = se[i];
    a.eigr[i] = sd[i];
    if (a.eigi) a.eigi[i] = 0.0;
  }
  if (!mem.inplace)
    for (int i = tid; i < n * n; i += DS_THREADS) a.Q[(i % n) + (size_t)(i / n) * a.ld] = Qs[i];
  if (tid == 0 && (flags & DS_DO_CONTROL)) {
    // EPSKrylovConvergence: first index from nconv whose estimate fails
    int kk;
    for (kk = l; kk < n; ++kk) {
      a.errest[kk] = serr[kk];
      if (serr[kk] >= a.tol) break;
    }
    for (int i = kk + 1; i < n; ++i) a.errest[i] = serr[i];
    KSControl *ctl = a.ctl;
    int reason = 0;
    if (kk >= a.nev) reason = 1;
    else if (a.its >= a.max_it) reason = -1;
    const int breakdown = st->breakdown;
    int lkeep;
    if (reason != 0 || breakdown || kk == n) lkeep = 0;
    else {
      lkeep = (int)((n - kk) * a.keep);
      if (lkeep < 1) lkeep = 1;
    }
    if (!a.lock && lkeep > 0) { lkeep += kk; kk = 0; }
    ctl->nconv = kk;
    ctl->l = lkeep;
    ctl->reason = reason;
    ctl->nv = n;
    ctl->breakdown = breakdown;
    ctl->need_start = (reason == 0 && (breakdown || kk == n) && kk < a.nev) ? 1 : 0;
    ctl->ds_error = s_fail;
    ctl->beta = beta;
  }
}

__global__ void __launch_bounds__(DS_THREADS, 1) k_ds_hep(DSArgs a) {
  extern __shared__ double Qs[];
  if (a.run_if && *a.run_if == 0) return;  // the fallback of the mixed-precision solver, not needed this restart
  DS_SMALL_MEM(m, Qs, 0);
  ds_hep_body(a, m);
}

// projected problems above 144: Q rotated in place in the caller's array, per-index scratch in dynamic shared memory
__global__ void __launch_bounds__(DS_THREADS, 1) k_ds_hep_wide(DSArgs a) {
  extern __shared__ __align__(16) unsigned char dsraw[];
  const int n = a.st ? a.st->m : a.n;
  ds_hep_body(a, ds_wide_mem(dsraw, n, a.Q, a.ld));
}

// one block per instance of a batch whose projected problem is symmetric (grid-stride over the live list)
__global__ void __launch_bounds__(DS_THREADS) k_batch_ds_hep(const BatchInst *I, const int *list, const BatchHdr *h) {
  extern __shared__ double Qs[];
  for (int v = blockIdx.x; v < h->n_inst; v += gridDim.x) {
    const BatchInst &p = I[list[v]];
    if (p.phase != BP_ITER || !p.hermitian) continue;
    __syncthreads();
    DS_SMALL_MEM(m, Qs, 0);
    ds_hep_body(batch_ds_args(p), m);
  }
}

cudaError_t batch_prepare_ds_hep(int max_ld) {
  if (max_ld > DS_MAXN) return cudaErrorInvalidValue;
  return cudaFuncSetAttribute(k_batch_ds_hep, cudaFuncAttributeMaxDynamicSharedMemorySize, max_ld * max_ld * 8);
}

cudaError_t launch_batch_ds_hep(const BatchInst *I, const int *list, const BatchHdr *h, int grid, int max_ld,
                                cudaStream_t s) {
  if (max_ld > DS_MAXN) return cudaErrorInvalidValue;
  k_batch_ds_hep<<<grid, DS_THREADS, (size_t)max_ld * max_ld * 8, s>>>(I, list, h);
  return cudaGetLastError();
}

int ds_hep_max_n() { return DS_WIDE_MAXN; }

cudaError_t launch_ds_hep(const DSArgs &a, int n_max, cudaStream_t s) {
  if (n_max > DS_WIDE_MAXN || a.ld < n_max) return cudaErrorInvalidValue;
  if (n_max > DS_MAXN) {
    const size_t shm = ds_wide_smem(n_max);
    cudaError_t err = cudaFuncSetAttribute(k_ds_hep_wide, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm);
    if (err != cudaSuccess) return err;
    k_ds_hep_wide<<<1, DS_THREADS, shm, s>>>(a);
    return cudaGetLastError();
  }
  const size_t shm = (size_t)n_max * n_max * 8;
  cudaError_t err = cudaFuncSetAttribute(k_ds_hep, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm);
  if (err != cudaSuccess) return err;
  k_ds_hep<<<1, DS_THREADS, shm, s>>>(a);
  return cudaGetLastError();
}

}  // namespace ksg
