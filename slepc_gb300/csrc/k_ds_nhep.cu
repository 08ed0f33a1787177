// k_ds_nhep.cu -- projected problem of the non-symmetric Krylov-Schur iteration, solved on the device in FP64.
//
// One 128-thread block per projected problem (thread 0 or warp 0 runs the scalar recurrences, the block applies the
// transformations), so the same code serves the single large solve and many small solves side by side.  It follows
// the reference's DSNHEP path:
//   DSSolve_NHEP_Private (src/sys/classes/ds/impls/dsutil.c:21-87): Householder reduction to Hessenberg form of the
//     rows/columns from l on (gehrd with ILO = l+1) when the matrix holds the Krylov-Schur form, then the real
//     Schur form by Francis double-shift QR (the algorithm of hseqr/lahqr) with standardised 2x2 blocks (lanv2);
//   DSSort_NHEP_Total (dsutil.c:93-171): selection sort by the criterion, moving blocks by direct swapping of
//     adjacent Schur blocks (Bai and Demmel 1993, the algorithm of trexc/laexc);
//   DSUpdateExtraRow_NHEP (dsnhep.c:318-340), DSVectors_NHEP_Eigen_Some (dsnhep.c:101-166) for the residual
//     estimates of EPSKrylovConvergence (epskrylov.c:207-295), DSGetTruncateSize (dsops.c:329-344) and
//     DSTruncate_NHEP (dsnhep.c:394-425).
// The solver is a long chain of short FP64 steps (one bulge reflector, then its application), and one warp issues
// FP64 instructions at a fraction of the SM's rate: four warps, one per SM sub-partition, apply each transformation
// together, and every thread computes the small reflectors itself instead of waiting for a broadcast.  A (and Q,
// when both fit) are staged in shared memory with odd strides, so threads walking rows or columns of a
// column-major array hit distinct banks.
#include <float.h>

#include "batch_types.h"
#include "common.cuh"
#include "kernels.h"
#include "ks_types.h"

namespace ksg {

constexpr int NH_MAXN = 144;
constexpr int NH_WIDE_MAXN = 640;  // the wide solver: A and Q in the caller's arrays (global memory, L2-resident)
constexpr int NH_T = 128;  // threads of one solver: four warps, one per SM sub-partition (each has its own FP64 pipe)

constexpr int NH_SMEM_MAX = 220 * 1024;  // dynamic shared memory of one solver (A, and Q when both fit)

#define AH(i, j) A[(i) + (size_t)(j) * lda]
#define QH(i, j) Q[(i) + (size_t)(j) * ldq]

template <int MAXN>
struct NhShared {
  double v[MAXN + 4];
  double G[16];
  double red[NH_T / 32];
  double tau, beta, cs, sn;
  double rf[2][4];  // bulge-chase reflectors (tau, v1, v2) of steps k and k+1
  double pc[MAXN / 2 + 1], ps[MAXN / 2 + 1];  // Givens rotations of one round of the parallel sort
  int pf[MAXN / 2 + 1];
  int cmd, i0, i1, i2, i3;
  int fail;
};

// odd strides >= rows: consecutive columns of a column-major array start in distinct banks
KS_DEVICE int nh_stride_a(int n) { return (n + 1) | 1; }  // A holds rows 0..n (the extra row n)
KS_DEVICE int nh_stride_q(int n) { return n | 1; }
__host__ __device__ inline size_t nh_smem_a(int n) { return (size_t)((n + 1) | 1) * n * sizeof(double); }
__host__ __device__ inline size_t nh_smem_q(int n) { return (size_t)(n | 1) * n * sizeof(double); }

KS_DEVICE int lane_id() { return threadIdx.x & 31; }
KS_DEVICE int nh_tid() { return threadIdx.x; }
KS_DEVICE void nh_sync() { __syncthreads(); }

// Householder vector of x[0..m-1] (one thread): x becomes v with v[0] = 1; returns tau, *beta = resulting head.
// H = I - tau v v^T maps x to (beta, 0, ..., 0) (the convention of LAPACK's larfg).  The norm is a plain sum of
// squares and one square root; the scaled sum (no divisions on the common path otherwise) is used only when the
// squares leave the safe range.
__device__ double nh_house_scaled(int m, double *x, double *beta) {
  const double alpha = x[0];
  double scale = 0.0, ssq = 1.0;
  for (int i = 1; i < m; ++i) {
    if (x[i] != 0.0) {
      const double a = fabs(x[i]);
      if (scale < a) {
        ssq = 1.0 + ssq * (scale / a) * (scale / a);
        scale = a;
      } else ssq += (a / scale) * (a / scale);
    }
  }
  const double xn = scale * sqrt(ssq);
  if (xn == 0.0) {
    *beta = alpha;
    x[0] = 1.0;
    return 0.0;
  }
  const double b = -copysign(hypot(alpha, xn), alpha);
  const double tau = (b - alpha) / b;
  const double sc = 1.0 / (alpha - b);
  for (int i = 1; i < m; ++i) x[i] *= sc;
  x[0] = 1.0;
  *beta = b;
  return tau;
}

constexpr double NH_SQ_LO = 1e-280, NH_SQ_HI = 1e280;

__device__ double nh_house(int m, double *x, double *beta) {
  const double alpha = x[0];
  double s2 = 0.0;
  for (int i = 1; i < m; ++i) s2 = fma(x[i], x[i], s2);
  const double t = fma(alpha, alpha, s2);
  if (s2 == 0.0 || t < NH_SQ_LO || t > NH_SQ_HI) return nh_house_scaled(m, x, beta);
  const double b = -copysign(sqrt(t), alpha);
  const double tau = (b - alpha) / b;
  const double sc = 1.0 / (alpha - b);
  for (int i = 1; i < m; ++i) x[i] *= sc;
  x[0] = 1.0;
  *beta = b;
  return tau;
}

KS_DEVICE double warp_sum_all(double v) {
  // butterfly: every lane ends with the same bits (each level adds the same two operands on both partners)
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// sum over the block, the same bits in every thread (warp butterflies, then the warp sums in a fixed order)
KS_DEVICE double nh_block_sum(double v, double *red) {
  v = warp_sum_all(v);
  if (lane_id() == 0) red[threadIdx.x >> 5] = v;
  nh_sync();
  double s = red[0];
  for (int w = 1; w < NH_T / 32; ++w) s += red[w];
  nh_sync();
  return s;
}

// the reflector of a long vector computed by the whole block (x in shared memory, the Hessenberg reduction);
// every thread returns tau, sh.beta holds beta
template <class SH>
__device__ double nh_house_block(int m, double *x, SH &sh) {
  const int tid = nh_tid();
  double s2 = 0.0;
  for (int i = 1 + tid; i < m; i += NH_T) s2 = fma(x[i], x[i], s2);
  s2 = nh_block_sum(s2, sh.red);
  const double alpha = x[0];
  const double t = fma(alpha, alpha, s2);
  if (s2 == 0.0 || t < NH_SQ_LO || t > NH_SQ_HI) {
    if (tid == 0) {
      double beta;
      sh.tau = nh_house_scaled(m, x, &beta);
      sh.beta = beta;
    }
    nh_sync();
    return sh.tau;
  }
  const double b = -copysign(sqrt(t), alpha);
  const double tau = (b - alpha) / b;
  const double sc = 1.0 / (alpha - b);
  for (int i = 1 + tid; i < m; i += NH_T) x[i] *= sc;
  if (tid == 0) {
    x[0] = 1.0;
    sh.beta = b;
  }
  nh_sync();
  return tau;
}

// block-parallel reflector applications (v, tau in shared memory); long dot products use four partial sums
__device__ void nh_refl_left(double *A, int lda, int r0, int m, int c0, int c1, const double *v, double tau) {
  for (int j = c0 + nh_tid(); j <= c1; j += NH_T) {
    double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
    int i = 0;
    for (; i + 3 < m; i += 4) {
      s0 = fma(v[i], AH(r0 + i, j), s0);
      s1 = fma(v[i + 1], AH(r0 + i + 1, j), s1);
      s2 = fma(v[i + 2], AH(r0 + i + 2, j), s2);
      s3 = fma(v[i + 3], AH(r0 + i + 3, j), s3);
    }
    for (; i < m; ++i) s0 = fma(v[i], AH(r0 + i, j), s0);
    const double s = ((s0 + s1) + (s2 + s3)) * tau;
    for (int i2 = 0; i2 < m; ++i2) AH(r0 + i2, j) -= s * v[i2];
  }
}
__device__ void nh_refl_right(double *A, int lda, int c0, int m, int r0, int r1, const double *v, double tau) {
  for (int i = r0 + nh_tid(); i <= r1; i += NH_T) {
    double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
    int j = 0;
    for (; j + 3 < m; j += 4) {
      s0 = fma(AH(i, c0 + j), v[j], s0);
      s1 = fma(AH(i, c0 + j + 1), v[j + 1], s1);
      s2 = fma(AH(i, c0 + j + 2), v[j + 2], s2);
      s3 = fma(AH(i, c0 + j + 3), v[j + 3], s3);
    }
    for (; j < m; ++j) s0 = fma(AH(i, c0 + j), v[j], s0);
    const double s = ((s0 + s1) + (s2 + s3)) * tau;
    for (int j2 = 0; j2 < m; ++j2) AH(i, c0 + j2) -= s * v[j2];
  }
}
// BLAS rot on rows (x: row p, y: row p+1, columns c0..c1) or columns (rows r0..r1)
__device__ void nh_rot_rows(double *A, int lda, int p, int c0, int c1, double c, double s) {
  for (int j = c0 + nh_tid(); j <= c1; j += NH_T) {
    const double x = AH(p, j), y = AH(p + 1, j);
    AH(p, j) = c * x + s * y;
    AH(p + 1, j) = c * y - s * x;
  }
}
__device__ void nh_rot_cols(double *A, int lda, int p, int r0, int r1, double c, double s) {
  for (int i = r0 + nh_tid(); i <= r1; i += NH_T) {
    const double x = AH(i, p), y = AH(i, p + 1);
    AH(i, p) = c * x + s * y;
    AH(i, p + 1) = c * y - s * x;
  }
}

// 2x2 standardisation (one thread): [a b; c d] -> G^T [a b; c d] G, G = [cs -sn; sn cs]
__device__ void nh_std2x2(double &a, double &b, double &c, double &d, double &cs, double &sn) {
  const double eps = DBL_EPSILON;
  if (c == 0.0) { cs = 1.0; sn = 0.0; return; }
  if (b == 0.0) {
    cs = 0.0; sn = 1.0;
    const double t = d; d = a; a = t; b = -c; c = 0.0;
    return;
  }
  if ((a - d) == 0.0 && copysign(1.0, b) != copysign(1.0, c)) { cs = 1.0; sn = 0.0; return; }
  double temp = a - d;
  double p = 0.5 * temp;
  const double bcmax = fmax(fabs(b), fabs(c));
  const double bcmis = fmin(fabs(b), fabs(c)) * copysign(1.0, b) * copysign(1.0, c);
  const double scale = fmax(fabs(p), bcmax);
  double z = (p / scale) * p + (bcmax / scale) * bcmis;
  if (z >= 4.0 * eps) {
    z = p + copysign(sqrt(scale) * sqrt(z), p);
    a = d + z;
    d = d - (bcmax / z) * bcmis;
    const double tau = hypot(c, z);
    cs = z / tau;
    sn = c / tau;
    b = b - c;
    c = 0.0;
  } else {
    const double sigma = b + c;
    const double tau = hypot(sigma, temp);
    cs = sqrt(0.5 * (1.0 + fabs(sigma) / tau));
    sn = -(p / (tau * cs)) * copysign(1.0, sigma);
    const double aa = a * cs + b * sn, bb = -a * sn + b * cs;
    const double cc = c * cs + d * sn, dd = -c * sn + d * cs;
    a = aa * cs + cc * sn;
    b = bb * cs + dd * sn;
    c = -aa * sn + cc * cs;
    d = -bb * sn + dd * cs;
    temp = 0.5 * (a + d);
    a = temp;
    d = temp;
    if (c != 0.0) {
      if (b != 0.0) {
        if (copysign(1.0, b) == copysign(1.0, c)) {
          const double sab = sqrt(fabs(b)), sac = sqrt(fabs(c));
          p = copysign(sab * sac, c);
          const double tau2 = 1.0 / sqrt(fabs(b + c));
          a = temp + p;
          d = temp - p;
          b = b - c;
          c = 0.0;
          const double cs1 = sab * tau2, sn1 = sac * tau2;
          temp = cs * cs1 - sn * sn1;
          sn = cs * sn1 + sn * cs1;
          cs = temp;
        }
      } else {
        b = -c;
        c = 0.0;
        temp = cs;
        cs = -sn;
        sn = temp;
      }
    }
  }
}

// standardise the 2x2 block at (i, i+1) and propagate to T and Q (whole block)
template <class SH>
__device__ void nh_std_block(double *A, int lda, double *Q, int ldq, int n, int i, SH &sh) {
  if (nh_tid() == 0) {
    double a = AH(i, i), b = AH(i, i + 1), c = AH(i + 1, i), d = AH(i + 1, i + 1), cs, sn;
    nh_std2x2(a, b, c, d, cs, sn);
    AH(i, i) = a; AH(i, i + 1) = b; AH(i + 1, i) = c; AH(i + 1, i + 1) = d;
    sh.cs = cs;
    sh.sn = sn;
  }
  nh_sync();
  const double cs = sh.cs, sn = sh.sn;
  if (i + 2 < n) nh_rot_rows(A, lda, i, i + 2, n - 1, cs, sn);
  if (i > 0) nh_rot_cols(A, lda, i, 0, i - 1, cs, sn);
  nh_rot_cols(Q, ldq, i, 0, n - 1, cs, sn);
  nh_sync();
}

// Hessenberg reduction from column ilo (rows/columns before ilo already triangular), accumulated into Q
template <class SH>
__device__ void nh_hessenberg(double *A, int lda, double *Q, int ldq, int n, int ilo, SH &sh) {
  for (int c = ilo; c < n - 2; ++c) {
    const int m = n - c - 1;
    for (int i = nh_tid(); i < m; i += NH_T) sh.v[i] = AH(c + 1 + i, c);
    nh_sync();
    const double tau = nh_house_block(m, sh.v, sh);
    if (tau != 0.0) {
      nh_refl_left(A, lda, c + 1, m, c + 1, n - 1, sh.v, tau);
      nh_sync();
      nh_refl_right(A, lda, c + 1, m, 0, n - 1, sh.v, tau);
      nh_refl_right(Q, ldq, c + 1, m, 0, n - 1, sh.v, tau);
      nh_sync();
      for (int i = nh_tid(); i < m; i += NH_T) AH(c + 1 + i, c) = i ? 0.0 : sh.beta;
    }
    nh_sync();
  }
}

// deflation test of the double-shift QR (lahqr) for the subdiagonal entry H(l, l-1), ilo < l <= ihi
KS_DEVICE bool nh_negligible(const double *A, int lda, int l, int ilo, int ihi, double smlnum) {
  const double eps = DBL_EPSILON;
  const double hll = fabs(AH(l, l - 1));
  if (hll <= smlnum) return true;
  double tst = fabs(AH(l - 1, l - 1)) + fabs(AH(l, l));
  if (tst == 0.0) {
    if (l - 2 >= ilo) tst += fabs(AH(l - 1, l - 2));
    if (l + 1 <= ihi) tst += fabs(AH(l + 1, l));
  }
  if (hll <= eps * tst) {
    const double ab = fmax(hll, fabs(AH(l - 1, l)));
    const double ba = fmin(hll, fabs(AH(l - 1, l)));
    const double aa = fmax(fabs(AH(l, l)), fabs(AH(l - 1, l - 1) - AH(l, l)));
    const double bb = fmin(fabs(AH(l, l)), fabs(AH(l - 1, l - 1) - AH(l, l)));
    const double s = aa + ab;
    if (ba * (ab / s) <= fmax(smlnum, eps * (bb * (aa / s)))) return true;
  }
  return false;
}

// reflector of (x0, x1, x2) with v = (1, v1, v2) (x2 = 0 for a 2-element reflector), computed identically by every
// thread from the same inputs
// With r = 1/sqrt(t), t = x0^2 + x1^2 + x2^2: beta = -sign(x0) t r, tau = (beta - x0)/beta = 1 + |x0| r, and the
// vector scale 1/(x0 - beta) = sign(x0)/(|x0| + t r): one reciprocal square root and one reciprocal.  The range
// tests read the bit pattern of t (non-negative doubles order as integers).
KS_DEVICE void nh_house3(double x0, double x1, double x2, double &tau, double &v1, double &v2, double &beta) {
  const double s2 = fma(x2, x2, x1 * x1);
  const double t = fma(x0, x0, s2);
  const long long tb = __double_as_longlong(t);
  if (__double_as_longlong(s2) == 0 || tb < __double_as_longlong(NH_SQ_LO) || tb > __double_as_longlong(NH_SQ_HI)) {
    double x[3] = {x0, x1, x2};
    tau = nh_house_scaled(3, x, &beta);
    v1 = x[1];
    v2 = x[2];
    return;
  }
  const double r = rsqrt(t);
  const double root = t * r;
  const double ax0 = fabs(x0);
  beta = copysign(root, -x0);
  tau = fma(ax0, r, 1.0);
  const double sc = copysign(__drcp_rn(ax0 + root), x0);
  v1 = x1 * sc;
  v2 = x2 * sc;
}

// Real Schur form of the Hessenberg matrix (rows/columns before ilo triangular) by the double-shift QR algorithm
// (lahqr: deflation test, exceptional shifts at 10 and 20 iterations, bulge chase with 3-element reflectors);
// returns 0 or 1 (no convergence).  Warp 0 runs the deflation scan (32 subdiagonals per ballot) and the shift
// computation in lockstep, every thread computes each bulge reflector, and the block applies it.
template <class SH>
__device__ int nh_francis(double *A, int lda, double *Q, int ldq, int n, int ilo, SH &sh) {
  const double smlnum = DBL_MIN * ((double)n / DBL_EPSILON);
  const int tid = nh_tid();
  for (int i = ilo + 2 + tid; i < n; i += NH_T)
    for (int j = ilo; j < i - 1; ++j) AH(i, j) = 0.0;
  nh_sync();
  int ihi = n - 1, its = 0, totits = 0;  // warp 0's copies (the same in every lane)
  const int maxtot = 40 * (n > 10 ? n : 10);
  for (;;) {
    if (tid < 32) {
      int cmd = 0, i0 = 0, i1 = 0, fail = 0;
      double v0 = 0.0, v1 = 0.0, v2 = 0.0;
      while (ihi >= ilo) {
        // the largest l in (ilo, ihi] whose subdiagonal is negligible, else ilo
        int l = ilo;
        for (int top = ihi; top > ilo; top -= 32) {
          const int cand = top - tid;
          const bool ok = cand > ilo && nh_negligible(A, lda, cand, ilo, ihi, smlnum);
          const unsigned bal = __ballot_sync(0xffffffffu, ok);
          if (bal) {
            l = top - (__ffs(bal) - 1);
            break;
          }
        }
        if (l > ilo && tid == 0) AH(l, l - 1) = 0.0;
        __syncwarp();
        if (l >= ihi) {
          ihi -= 1;
          its = 0;
          continue;
        }
        if (l == ihi - 1) {
          cmd = 1;
          i0 = l;
          ihi -= 2;
          its = 0;
          break;
        }
        if (++totits > maxtot) {
          fail = 1;
          break;
        }
        its++;
        double h11, h12, h21, h22;
        if (its == 10) {
          const double s = fabs(AH(l + 1, l)) + fabs(AH(l + 2, l + 1));
          h11 = 0.75 * s + AH(l, l);
          h12 = -0.4375 * s;
          h21 = s;
          h22 = h11;
        } else if (its == 20) {
          const double s = fabs(AH(ihi, ihi - 1)) + fabs(AH(ihi - 1, ihi - 2));
          h11 = 0.75 * s + AH(ihi, ihi);
          h12 = -0.4375 * s;
          h21 = s;
          h22 = h11;
        } else {
          h11 = AH(ihi - 1, ihi - 1);
          h21 = AH(ihi, ihi - 1);
          h12 = AH(ihi - 1, ihi);
          h22 = AH(ihi, ihi);
        }
        const double s = fabs(h11) + fabs(h12) + fabs(h21) + fabs(h22);
        double rt1r, rt1i, rt2r, rt2i;
        if (s == 0.0) {
          rt1r = rt1i = rt2r = rt2i = 0.0;
        } else {
          h11 /= s; h21 /= s; h12 /= s; h22 /= s;
          const double tr = (h11 + h22) / 2.0;
          const double det = (h11 - tr) * (h22 - tr) - h12 * h21;
          const double rtdisc = sqrt(fabs(det));
          if (det >= 0.0) {
            rt1r = tr * s; rt2r = rt1r; rt1i = rtdisc * s; rt2i = -rt1i;
          } else {
            rt1r = tr + rtdisc;
            rt2r = tr - rtdisc;
            if (fabs(rt1r - h22) <= fabs(rt2r - h22)) { rt1r *= s; rt2r = rt1r; }
            else { rt2r *= s; rt1r = rt2r; }
            rt1i = rt2i = 0.0;
          }
        }
        const int m = l;
        double h21s = AH(m + 1, m);
        double sc = fabs(AH(m, m) - rt2r) + fabs(rt2i) + fabs(h21s);
        h21s /= sc;
        const double w0 = h21s * AH(m, m + 1) + (AH(m, m) - rt1r) * ((AH(m, m) - rt2r) / sc) - rt1i * (rt2i / sc);
        const double w1 = h21s * (AH(m, m) + AH(m + 1, m + 1) - rt1r - rt2r);
        const double w2 = h21s * AH(m + 2, m + 1);
        sc = fabs(w0) + fabs(w1) + fabs(w2);
        v0 = w0 / sc;
        v1 = w1 / sc;
        v2 = w2 / sc;
        cmd = 2;
        i0 = m;
        i1 = ihi;
        break;
      }
      if (tid == 0) {
        sh.cmd = cmd;
        sh.i0 = i0;
        sh.i1 = i1;
        sh.v[0] = v0;
        sh.v[1] = v1;
        sh.v[2] = v2;
        if (fail) sh.fail = 1;
      }
    }
    nh_sync();
    const int cmd = sh.cmd;
    if (cmd == 0) break;
    if (cmd == 1) {
      nh_std_block(A, lda, Q, ldq, n, sh.i0, sh);
      continue;
    }
    // bulge chase over [m, hi].  Warp 0 owns the critical path of each step: the update of the 4 x 3 block that
    // the next reflector depends on (rows k..k+3, columns k..k+2, both sides), then that reflector and the zeros
    // of its column; warps 1-3 meanwhile apply the step to the rest of A (the rows' remaining columns, the
    // columns' rows above k) and to Q.  The regions are disjoint, so one barrier per step suffices, and every
    // entry gets the same operations as in a block-wide update.
    const int m = sh.i0, hi = sh.i1;
    const int warp = tid >> 5, lane = tid & 31;
    if (warp == 0) {
      const int nr = (3 < hi - m + 1) ? 3 : hi - m + 1;
      double tau, v1, v2, beta;
      nh_house3(sh.v[0], sh.v[1], nr == 3 ? sh.v[2] : 0.0, tau, v1, v2, beta);
      if (lane == 0) {
        sh.rf[m & 1][0] = tau;
        sh.rf[m & 1][1] = v1;
        sh.rf[m & 1][2] = v2;
      }
    }
    nh_sync();
    for (int k = m; k <= hi - 1; ++k) {
      const int nr = (3 < hi - k + 1) ? 3 : hi - k + 1;
      const int cb = k + nr;                    // first column right of the reflector's
      const int r1 = (k + 3 < hi) ? k + 3 : hi;  // last row the column update reaches
      const double tau = sh.rf[k & 1][0], v1 = sh.rf[k & 1][1], v2 = sh.rf[k & 1][2];
      if (tau != 0.0) {  // else x was already (x0, 0, 0): nothing changes
        const double w0 = tau, w1 = tau * v1, w2 = tau * v2;
        if (warp == 0) {
          // rows k..k+nr-1 over the block's columns k..cb-1
          if (lane < nr) {
            const int j = k + lane;
            const double a0 = AH(k, j), a1 = AH(k + 1, j);
            if (nr == 3) {
              const double a2 = AH(k + 2, j);
              const double d = fma(v2, a2, fma(v1, a1, a0));
              AH(k, j) = fma(-d, w0, a0);
              AH(k + 1, j) = fma(-d, w1, a1);
              AH(k + 2, j) = fma(-d, w2, a2);
            } else {
              const double d = fma(v1, a1, a0);
              AH(k, j) = fma(-d, w0, a0);
              AH(k + 1, j) = fma(-d, w1, a1);
            }
          }
          __syncwarp();
          // columns k..cb-1 over the block's rows k..r1
          if (lane <= r1 - k) {
            double *row = A + (k + lane);
            const double a0 = row[(size_t)k * lda], a1 = row[(size_t)(k + 1) * lda];
            if (nr == 3) {
              const double a2 = row[(size_t)(k + 2) * lda];
              const double d = fma(a2, v2, fma(a1, v1, a0));
              row[(size_t)k * lda] = fma(-d, w0, a0);
              row[(size_t)(k + 1) * lda] = fma(-d, w1, a1);
              row[(size_t)(k + 2) * lda] = fma(-d, w2, a2);
            } else {
              const double d = fma(a1, v1, a0);
              row[(size_t)k * lda] = fma(-d, w0, a0);
              row[(size_t)(k + 1) * lda] = fma(-d, w1, a1);
            }
          }
          __syncwarp();
        } else {
          const int bt = tid - 32;
          constexpr int NB = NH_T - 32;
          // rows k..k+nr-1 over columns cb..n-1
          for (int j = cb + bt; j < n; j += NB) {
            const double a0 = AH(k, j), a1 = AH(k + 1, j);
            if (nr == 3) {
              const double a2 = AH(k + 2, j);
              const double d = fma(v2, a2, fma(v1, a1, a0));
              AH(k, j) = fma(-d, w0, a0);
              AH(k + 1, j) = fma(-d, w1, a1);
              AH(k + 2, j) = fma(-d, w2, a2);
            } else {
              const double d = fma(v1, a1, a0);
              AH(k, j) = fma(-d, w0, a0);
              AH(k + 1, j) = fma(-d, w1, a1);
            }
          }
          // columns k..cb-1 over rows 0..k-1 of the matrix and all rows of the Schur vectors
          for (int t = bt; t < k + n; t += NB) {
            double *row;
            int ldm;
            if (t < k) { row = A + t; ldm = lda; }
            else { row = Q + (t - k); ldm = ldq; }
            const double a0 = row[(size_t)k * ldm], a1 = row[(size_t)(k + 1) * ldm];
            if (nr == 3) {
              const double a2 = row[(size_t)(k + 2) * ldm];
              const double d = fma(a2, v2, fma(a1, v1, a0));
              row[(size_t)k * ldm] = fma(-d, w0, a0);
              row[(size_t)(k + 1) * ldm] = fma(-d, w1, a1);
              row[(size_t)(k + 2) * ldm] = fma(-d, w2, a2);
            } else {
              const double d = fma(a1, v1, a0);
              row[(size_t)k * ldm] = fma(-d, w0, a0);
              row[(size_t)(k + 1) * ldm] = fma(-d, w1, a1);
            }
          }
        }
      }
      if (warp == 0 && k + 1 <= hi - 1) {
        // the next step's reflector from column k, which becomes (beta, 0, 0): no other warp touches those
        // entries in this step or the next
        const int nr1 = (3 < hi - k) ? 3 : hi - k;
        const double y0 = AH(k + 1, k), y1 = AH(k + 2, k), y2 = nr1 == 3 ? AH(k + 3, k) : 0.0;
        double t1, u1, u2, b1;
        nh_house3(y0, y1, y2, t1, u1, u2, b1);
        __syncwarp();  // every lane has read column k
        if (lane == 0) {
          sh.rf[(k + 1) & 1][0] = t1;
          sh.rf[(k + 1) & 1][1] = u1;
          sh.rf[(k + 1) & 1][2] = u2;
          if (t1 != 0.0) {
            AH(k + 1, k) = b1;
            AH(k + 2, k) = 0.0;
            if (nr1 == 3) AH(k + 3, k) = 0.0;
          }
        }
      }
      nh_sync();
    }
  }
  return sh.fail;
}

// small Sylvester solve T11 X - X T22 = B (Kronecker system, complete pivoting), one thread
__device__ void nh_sylv(int n1, int n2, const double *D, double *X, double smin) {
  const int m = n1 * n2;
  double K[4][4], rhs[4];
  int colp[4];
  for (int i = 0; i < m; ++i)
    for (int j = 0; j < m; ++j) K[i][j] = 0.0;
  for (int c = 0; c < n2; ++c)
    for (int r = 0; r < n1; ++r) {
      const int u = r + c * n1;
      rhs[u] = D[r + (n1 + c) * 4];
      for (int k = 0; k < n1; ++k) K[u][k + c * n1] += D[r + k * 4];
      for (int k = 0; k < n2; ++k) K[u][r + k * n1] -= D[(n1 + k) + (n1 + c) * 4];
    }
  for (int i = 0; i < m; ++i) colp[i] = i;
  for (int p = 0; p < m; ++p) {
    int bi = p, bj = p;
    double best = -1.0;
    for (int i = p; i < m; ++i)
      for (int j = p; j < m; ++j)
        if (fabs(K[i][j]) > best) { best = fabs(K[i][j]); bi = i; bj = j; }
    if (bi != p) {
      for (int j = 0; j < m; ++j) { const double t = K[p][j]; K[p][j] = K[bi][j]; K[bi][j] = t; }
      const double t = rhs[p]; rhs[p] = rhs[bi]; rhs[bi] = t;
    }
    if (bj != p) {
      for (int i = 0; i < m; ++i) { const double t = K[i][p]; K[i][p] = K[i][bj]; K[i][bj] = t; }
      const int t = colp[p]; colp[p] = colp[bj]; colp[bj] = t;
    }
    if (fabs(K[p][p]) < smin) K[p][p] = smin;
    for (int i = p + 1; i < m; ++i) {
      const double f = K[i][p] / K[p][p];
      for (int j = p; j < m; ++j) K[i][j] -= f * K[p][j];
      rhs[i] -= f * rhs[p];
    }
  }
  double y[4];
  for (int i = m - 1; i >= 0; --i) {
    double s = rhs[i];
    for (int j = i + 1; j < m; ++j) s -= K[i][j] * y[j];
    y[i] = s / K[i][i];
  }
  for (int i = 0; i < m; ++i) {
    const int u = colp[i];
    X[(u % n1) + (u / n1) * 2] = y[i];
  }
}

// swap adjacent blocks of sizes n1 (at j1) and n2 (at j1+n1); returns 1 if rejected
template <class SH>
__device__ int nh_swap(double *A, int lda, double *Q, int ldq, int n, int j1, int n1, int n2, SH &sh) {
  const int m = n1 + n2;
  if (n1 == 1 && n2 == 1) {
    const int j2 = j1 + 1;
    if (nh_tid() == 0) {
      const double t11 = AH(j1, j1), t22 = AH(j2, j2);
      const double f = AH(j1, j2), g = t22 - t11;
      double c, s;
      if (g == 0.0) { c = 1.0; s = 0.0; }
      else if (f == 0.0) { c = 0.0; s = copysign(1.0, g); }
      else {
        const double d = hypot(f, g);
        c = fabs(f) / d;
        s = g / copysign(d, f);
      }
      sh.cs = c;
      sh.sn = s;
      sh.G[0] = t11;
      sh.G[1] = t22;
    }
    nh_sync();
    const double c = sh.cs, s = sh.sn;
    if (j2 + 1 < n) nh_rot_rows(A, lda, j1, j2 + 1, n - 1, c, s);
    if (j1 > 0) nh_rot_cols(A, lda, j1, 0, j1 - 1, c, s);
    nh_rot_cols(Q, ldq, j1, 0, n - 1, c, s);
    nh_sync();
    if (nh_tid() == 0) {
      AH(j1, j1) = sh.G[1];
      AH(j2, j2) = sh.G[0];
    }
    nh_sync();
    return 0;
  }
  if (nh_tid() == 0) {
    const double eps = DBL_EPSILON;
    double D[16], dnorm = 0.0;
    for (int j = 0; j < m; ++j)
      for (int i = 0; i < m; ++i) {
        D[i + j * 4] = AH(j1 + i, j1 + j);
        dnorm = fmax(dnorm, fabs(D[i + j * 4]));
      }
    const double smin = fmax(eps * dnorm, DBL_MIN / eps);
    const double thresh = fmax(20.0 * eps * dnorm, DBL_MIN / eps);
    double X[4];
    nh_sylv(n1, n2, D, X, smin);
    double M[4][2];
    for (int c = 0; c < n2; ++c) {
      for (int r = 0; r < n1; ++r) M[r][c] = -X[r + c * 2];
      for (int r = 0; r < n2; ++r) M[n1 + r][c] = (r == c) ? 1.0 : 0.0;
    }
    double *G = sh.G;
    for (int i = 0; i < 16; ++i) G[i] = 0.0;
    for (int i = 0; i < m; ++i) G[i + i * 4] = 1.0;
    for (int c = 0; c < n2; ++c) {
      double v[4], beta;
      const int len = m - c;
      for (int i = 0; i < len; ++i) v[i] = M[c + i][c];
      const double tau = nh_house(len, v, &beta);
      if (tau == 0.0) continue;
      for (int cc = c; cc < n2; ++cc) {
        double s = 0.0;
        for (int i = 0; i < len; ++i) s += v[i] * M[c + i][cc];
        s *= tau;
        for (int i = 0; i < len; ++i) M[c + i][cc] -= s * v[i];
      }
      for (int i = 0; i < m; ++i) {
        double s = 0.0;
        for (int j = 0; j < len; ++j) s += G[i + (c + j) * 4] * v[j];
        s *= tau;
        for (int j = 0; j < len; ++j) G[i + (c + j) * 4] -= s * v[j];
      }
    }
    double W[16], D2[16];
    for (int i = 0; i < m; ++i)
      for (int j = 0; j < m; ++j) {
        double s = 0.0;
        for (int k = 0; k < m; ++k) s += D[i + k * 4] * G[k + j * 4];
        W[i + j * 4] = s;
      }
    for (int i = 0; i < m; ++i)
      for (int j = 0; j < m; ++j) {
        double s = 0.0;
        for (int k = 0; k < m; ++k) s += G[k + i * 4] * W[k + j * 4];
        D2[i + j * 4] = s;
      }
    double resid = 0.0;
    for (int i = n2; i < m; ++i)
      for (int j = 0; j < n2; ++j) resid = fmax(resid, fabs(D2[i + j * 4]));
    sh.cmd = resid > thresh;
  }
  nh_sync();
  if (sh.cmd) return 1;
  const double *G = sh.G;
  // left: rows j1..j1+m-1 over columns j1..n-1
  for (int j = j1 + nh_tid(); j < n; j += NH_T) {
    double t[4];
    for (int i = 0; i < m; ++i) {
      double s = 0.0;
      for (int k = 0; k < m; ++k) s += G[k + i * 4] * AH(j1 + k, j);
      t[i] = s;
    }
    for (int i = 0; i < m; ++i) AH(j1 + i, j) = t[i];
  }
  nh_sync();
  // right: columns j1..j1+m-1 over rows 0..j1+m-1; Q over all rows
  for (int i = nh_tid(); i < j1 + m; i += NH_T) {
    double t[4];
    for (int j = 0; j < m; ++j) {
      double s = 0.0;
      for (int k = 0; k < m; ++k) s += AH(i, j1 + k) * G[k + j * 4];
      t[j] = s;
    }
    for (int j = 0; j < m; ++j) AH(i, j1 + j) = t[j];
  }
  for (int i = nh_tid(); i < n; i += NH_T) {
    double t[4];
    for (int j = 0; j < m; ++j) {
      double s = 0.0;
      for (int k = 0; k < m; ++k) s += QH(i, j1 + k) * G[k + j * 4];
      t[j] = s;
    }
    for (int j = 0; j < m; ++j) QH(i, j1 + j) = t[j];
  }
  nh_sync();
  if (nh_tid() == 0)
    for (int i = n2; i < m; ++i)
      for (int j = 0; j < n2; ++j) AH(j1 + i, j1 + j) = 0.0;
  nh_sync();
  if (n2 == 2) nh_std_block(A, lda, Q, ldq, n, j1, sh);
  else {
    if (nh_tid() == 0) AH(j1 + 1, j1) = 0.0;
    nh_sync();
  }
  if (n1 == 2) nh_std_block(A, lda, Q, ldq, n, j1 + n2, sh);
  return 0;
}

// move the block at ifst up to ilst (ifst > ilst); 0 or 1 (rejected swap)
template <class SH>
__device__ int nh_move(double *A, int lda, double *Q, int ldq, int n, int ifst, int ilst, SH &sh) {
  if (ifst > 0 && AH(ifst, ifst - 1) != 0.0) ifst--;
  int nbf = (ifst < n - 1 && AH(ifst + 1, ifst) != 0.0) ? 2 : 1;
  if (ilst > 0 && AH(ilst, ilst - 1) != 0.0) ilst--;
  int here = ifst;
  while (here > ilst) {
    const int nbnext = (here >= 2 && AH(here - 1, here - 2) != 0.0) ? 2 : 1;
    if (nh_swap(A, lda, Q, ldq, n, here - nbnext, nbnext, nbf, sh)) return 1;
    nh_sync();
    if (nbf == 2 && AH(here - nbnext + 1, here - nbnext) == 0.0) nbf = 1;
    here -= nbnext;
  }
  return 0;
}

__device__ void nh_eigs(const double *A, int lda, int n, int from, double *wr, double *wi) {
  for (int j = from; j < n; ++j) {
    wr[j] = AH(j, j);
    if (j < n - 1 && AH(j + 1, j) != 0.0) {
      wi[j] = sqrt(fabs(AH(j + 1, j))) * sqrt(fabs(AH(j, j + 1)));
      wr[j + 1] = wr[j];
      wi[j + 1] = -wi[j];
      j++;
    } else wi[j] = 0.0;
  }
}

// right eigenvector of the quasi-triangular T for the block starting at k (single thread, trevc conventions)
__device__ int nh_eigvec(const double *A, int lda, int n, int k, double tnorm, double *xr, double *xi) {
  const double eps = DBL_EPSILON;
  const double smin = fmax(eps * tnorm, DBL_MIN / eps);
  for (int i = 0; i < n; ++i) { xr[i] = 0.0; xi[i] = 0.0; }
  const int cplx = (k < n - 1 && AH(k + 1, k) != 0.0);
  if (!cplx) {
    const double lam = AH(k, k);
    xr[k] = 1.0;
    double mx = 1.0;
    for (int i = k - 1; i >= 0; --i) {
      bool twice = false;  // a 2x2 block set xr[i-1] and xr[i]; i now indexes its first row
      if (i > 0 && AH(i, i - 1) != 0.0) {
        double r0 = 0.0, r1 = 0.0;
        for (int j = i + 1; j <= k; ++j) { r0 -= AH(i - 1, j) * xr[j]; r1 -= AH(i, j) * xr[j]; }
        const double a = AH(i - 1, i - 1) - lam, b = AH(i - 1, i), c = AH(i, i - 1), d = AH(i, i) - lam;
        double det = a * d - b * c;
        if (fabs(det) < smin) det = copysign(smin, det);
        xr[i - 1] = (r0 * d - b * r1) / det;
        xr[i] = (a * r1 - c * r0) / det;
        i--;
        twice = true;
      } else {
        double s = 0.0;
        for (int j = i + 1; j <= k; ++j) s -= AH(i, j) * xr[j];
        double den = AH(i, i) - lam;
        if (fabs(den) < smin) den = smin;
        xr[i] = s / den;
      }
      // max |xr[i..k]|, kept as a running maximum (entries below i are still zero)
      mx = fmax(mx, fabs(xr[i]));
      if (i + 1 <= k && twice) mx = fmax(mx, fabs(xr[i + 1]));
      if (mx > 1e150) {
        for (int j = 0; j <= k; ++j) xr[j] /= mx;
        mx = 0.0;
        for (int j = i; j <= k; ++j) mx = fmax(mx, fabs(xr[j]));
      }
    }
    return 0;
  }
  const int ki = k + 1;
  const double wr = AH(k, k);
  const double wim = sqrt(fabs(AH(k, ki))) * sqrt(fabs(AH(ki, k)));
  if (fabs(AH(k, ki)) >= fabs(AH(ki, k))) { xr[k] = 1.0; xi[ki] = wim / AH(k, ki); }
  else { xr[k] = -wim / AH(ki, k); xi[ki] = 1.0; }
  double mx = fmax(fabs(xr[k]) + fabs(xi[k]), fabs(xr[ki]) + fabs(xi[ki]));
  for (int i = k - 1; i >= 0; --i) {
    bool twice = false;
    if (i > 0 && AH(i, i - 1) != 0.0) {
      double r0r = 0.0, r0i = 0.0, r1r = 0.0, r1i = 0.0;
      for (int j = i + 1; j <= ki; ++j) {
        r0r -= AH(i - 1, j) * xr[j]; r0i -= AH(i - 1, j) * xi[j];
        r1r -= AH(i, j) * xr[j]; r1i -= AH(i, j) * xi[j];
      }
      const double ar = AH(i - 1, i - 1) - wr, ai = -wim, b = AH(i - 1, i);
      const double c = AH(i, i - 1), dr = AH(i, i) - wr, di = -wim;
      double detr = ar * dr - ai * di - b * c, deti = ar * di + ai * dr;
      double dd = detr * detr + deti * deti;
      if (dd < smin * smin) { detr = smin; deti = 0.0; dd = smin * smin; }
      double nr = r0r * dr - r0i * di - b * r1r, ni = r0r * di + r0i * dr - b * r1i;
      xr[i - 1] = (nr * detr + ni * deti) / dd;
      xi[i - 1] = (ni * detr - nr * deti) / dd;
      nr = ar * r1r - ai * r1i - c * r0r;
      ni = ar * r1i + ai * r1r - c * r0i;
      xr[i] = (nr * detr + ni * deti) / dd;
      xi[i] = (ni * detr - nr * deti) / dd;
      i--;
      twice = true;
    } else {
      double sr = 0.0, si = 0.0;
      for (int j = i + 1; j <= ki; ++j) { sr -= AH(i, j) * xr[j]; si -= AH(i, j) * xi[j]; }
      double denr = AH(i, i) - wr, deni = -wim;
      double dd = denr * denr + deni * deni;
      if (dd < smin * smin) { denr = smin; deni = 0.0; dd = smin * smin; }
      xr[i] = (sr * denr + si * deni) / dd;
      xi[i] = (si * denr - sr * deni) / dd;
    }
    // max |xr[j]| + |xi[j]| over j = i..ki, kept as a running maximum
    mx = fmax(mx, fabs(xr[i]) + fabs(xi[i]));
    if (twice) mx = fmax(mx, fabs(xr[i + 1]) + fabs(xi[i + 1]));
    if (mx > 1e150) {
      for (int j = 0; j <= ki; ++j) { xr[j] /= mx; xi[j] /= mx; }
      mx = 0.0;
      for (int j = i; j <= ki; ++j) mx = fmax(mx, fabs(xr[j]) + fabs(xi[j]));
    }
  }
  return 1;
}

// ordering of two eigenvalues by the criterion: > 0 when (r2, i2) goes before (r1, i1) (SlepcSCCompare, which
// values as in EPSWhich: 1 largest magnitude, 2 smallest magnitude, 3 largest real, 4 smallest real, 5 largest
// imaginary, 6 smallest imaginary, 7 closest to the target, 8 real part closest to the target; slepcsc.c:152-267)
KS_DEVICE int nh_cmp(int which, double target, double r1, double i1, double r2, double i2) {
  double av, bv;
  switch (which) {
    case 7: av = hypot(r1 - target, i1); bv = hypot(r2 - target, i2); return av > bv ? 1 : (av < bv ? -1 : 0);
    case 8: av = fabs(r1 - target); bv = fabs(r2 - target); return av > bv ? 1 : (av < bv ? -1 : 0);
    case 1: av = hypot(r1, i1); bv = hypot(r2, i2); return av < bv ? 1 : (av > bv ? -1 : 0);
    case 2: av = hypot(r1, i1); bv = hypot(r2, i2); return av > bv ? 1 : (av < bv ? -1 : 0);
    case 3: return r1 < r2 ? 1 : (r1 > r2 ? -1 : 0);
    case 4: return r1 > r2 ? 1 : (r1 < r2 ? -1 : 0);
    case 5: av = fabs(i1); bv = fabs(i2); return av < bv ? 1 : (av > bv ? -1 : 0);
    case 6: av = fabs(i1); bv = fabs(i2); return av > bv ? 1 : (av < bv ? -1 : 0);
    default: return 0;
  }
}

// Sort of a real Schur form with 1x1 blocks only (rows l..n-1) by odd-even transposition: in each round the
// out-of-order pairs (j, j+1) of one parity are exchanged by the 1x1 swap of the direct swapping method (a Givens
// rotation from T(j, j+1) and T(j+1, j+1) - T(j, j), trexc/laexc with n1 = n2 = 1).  Pairs of one round are
// disjoint, so their rotations commute: all row rotations are applied, then all column rotations (T and Q), then
// the diagonal exchanges.  The final order is the stable order of the criterion, as the selection sort's.
template <class SH>
__device__ void nh_sort_real(double *A, int lda, double *Q, int ldq, int n, int l, int which, double target,
                             double *wr, SH &sh) {
  const int tid = nh_tid();
  int quiet = 0;
  for (int round = 0; round < 2 * (n - l) + 2 && quiet < 2; ++round) {
    const int j0 = l + (round & 1);
    const int np = (n - j0) / 2;  // pairs (j0 + 2p, j0 + 2p + 1)
    int any = 0;
    for (int p = tid; p < np; p += NH_T) {
      const int j = j0 + 2 * p;
      const int sw = nh_cmp(which, target, wr[j], 0.0, wr[j + 1], 0.0) > 0;
      sh.pf[p] = sw;
      if (sw) {
        any = 1;
        const double t11 = AH(j, j), t22 = AH(j + 1, j + 1);
        const double f = AH(j, j + 1), g = t22 - t11;
        double c, sn;
        if (g == 0.0) { c = 1.0; sn = 0.0; }
        else if (f == 0.0) { c = 0.0; sn = copysign(1.0, g); }
        else {
          const double d = hypot(f, g);
          c = fabs(f) / d;
          sn = g / copysign(d, f);
        }
        sh.pc[p] = c;
        sh.ps[p] = sn;
      }
    }
    if (!__syncthreads_or(any)) {
      quiet++;
      continue;
    }
    quiet = 0;
    // rows j, j+1 over columns j+2..n-1
    for (int col = tid; col < n; col += NH_T)
      for (int p = 0; p < np; ++p) {
        const int j = j0 + 2 * p;
        if (j + 2 > col) break;
        if (!sh.pf[p]) continue;
        const double c = sh.pc[p], sn = sh.ps[p];
        const double x = AH(j, col), y = AH(j + 1, col);
        AH(j, col) = c * x + sn * y;
        AH(j + 1, col) = c * y - sn * x;
      }
    nh_sync();
    // columns j, j+1 over rows 0..j-1 of T (tasks 0..n-1) and over all rows of the Schur vectors (tasks n..2n-1)
    for (int t = tid; t < 2 * n; t += NH_T) {
      const bool isq = t >= n;
      const int r = isq ? t - n : t;
      double *row = isq ? Q + r : A + r;
      const int ldm = isq ? ldq : lda;
      for (int p = 0; p < np; ++p) {
        if (!sh.pf[p]) continue;
        const int j = j0 + 2 * p;
        if (!isq && r >= j) continue;
        const double c = sh.pc[p], sn = sh.ps[p];
        const double x = row[(size_t)j * ldm], y = row[(size_t)(j + 1) * ldm];
        row[(size_t)j * ldm] = c * x + sn * y;
        row[(size_t)(j + 1) * ldm] = c * y - sn * x;
      }
    }
    nh_sync();
    for (int p = tid; p < np; p += NH_T)
      if (sh.pf[p]) {
        const int j = j0 + 2 * p;
        const double t = AH(j, j);
        AH(j, j) = AH(j + 1, j + 1);
        AH(j + 1, j + 1) = t;
        const double w = wr[j];
        wr[j] = wr[j + 1];
        wr[j + 1] = w;
      }
    nh_sync();
  }
}

// Harmonic extraction, translation (DSTranslateHarmonic_NHEP, dsnhep.c:466-507): g = (A - tau I)^T \ (beta e_n)
// and A(:, n-1) += beta g; returns gamma = sqrt(1 + g'g), the correction factor of the residual estimates.  The
// reference factors A - tau I and solves with its transpose; here the transpose is copied into the scratch C
// (ldc >= n) and eliminated with partial pivoting (the row of largest magnitude, the first one on ties), which
// solves the same system.  A zero pivot (tau an eigenvalue of A) sets sh.fail.
template <class SH>
__device__ double nh_harmonic_translate(double *A, int lda, int n, double tau, double beta, double *C, int ldc,
                                        double *g, SH &sh) {
  const int tid = nh_tid();
  for (int t = tid; t < n * n; t += NH_T) {
    const int r = t % n, c = t / n;
    C[r + (size_t)c * ldc] = AH(c, r) - (r == c ? tau : 0.0);
  }
  for (int i = tid; i < n; i += NH_T) g[i] = (i == n - 1) ? beta : 0.0;
  nh_sync();
  for (int c = 0; c < n; ++c) {
    if (tid < 32) {
      double best = -1.0;
      int bi = c;
      for (int i = c + tid; i < n; i += 32) {
        const double v = fabs(C[i + (size_t)c * ldc]);
        if (v > best) { best = v; bi = i; }
      }
      for (int o = 16; o > 0; o >>= 1) {
        const double ob = __shfl_xor_sync(0xffffffffu, best, o);
        const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
        if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
      }
      if (tid == 0) {
        sh.i2 = bi;
        sh.tau = best;
      }
    }
    nh_sync();
    const int p = sh.i2;
    if (sh.tau == 0.0) {
      if (tid == 0) sh.fail = 3;
      nh_sync();
      return 1.0;
    }
    if (p != c) {
      for (int j = c + tid; j < n; j += NH_T) {
        const double t = C[c + (size_t)j * ldc];
        C[c + (size_t)j * ldc] = C[p + (size_t)j * ldc];
        C[p + (size_t)j * ldc] = t;
      }
      if (tid == 0) {
        const double t = g[c];
        g[c] = g[p];
        g[p] = t;
      }
      nh_sync();
    }
    const double piv = C[c + (size_t)c * ldc], gc = g[c];
    for (int i = c + 1 + tid; i < n; i += NH_T) {
      const double f = C[i + (size_t)c * ldc] / piv;
      for (int j = c + 1; j < n; ++j) C[i + (size_t)j * ldc] -= f * C[c + (size_t)j * ldc];
      g[i] -= f * gc;
    }
    nh_sync();
  }
  // back substitution, one column of U at a time
  for (int i = n - 1; i >= 0; --i) {
    if (tid == 0) g[i] /= C[i + (size_t)i * ldc];
    nh_sync();
    const double gi = g[i];
    for (int r = tid; r < i; r += NH_T) g[r] -= C[r + (size_t)i * ldc] * gi;
    nh_sync();
  }
  for (int i = tid; i < n; i += NH_T) AH(i, n - 1) += g[i] * beta;
  double s2 = 0.0;
  for (int i = tid; i < n; i += NH_T) s2 = fma(g[i], g[i], s2);
  s2 = nh_block_sum(s2, sh.red);
  return hypot(1.0, sqrt(s2));
}

// Harmonic extraction, recovery before the restart (dsnhep.c:508-535 with DSSetDimensions(n, k, l)):
// ghat = -Q(:, 0:k+l)^T g; A(i, j) += ghat_i Q(n-1, j) beta for i < k+l, k <= j < k+l; g <- g + Q(:, 0:k+l) ghat;
// gamma = sqrt(1 + g'g) scales the extra-row entries k..k+l-1.  Returns gamma; g holds g~.
template <class SH>
__device__ double nh_harmonic_recover(double *A, int lda, const double *Q, int ldq, int n, int k, int l,
                                      double beta, double *g, double *gh, SH &sh) {
  const int tid = nh_tid(), ncol = k + l;
  for (int j = tid; j < ncol; j += NH_T) {
    double s = 0.0;
    for (int i = 0; i < n; ++i) s = fma(QH(i, j), g[i], s);
    gh[j] = -s;
  }
  nh_sync();
  for (int t = tid; t < ncol * l; t += NH_T) {
    const int i = t % ncol, j = k + t / ncol;
    AH(i, j) += gh[i] * QH(n - 1, j) * beta;
  }
  for (int i = tid; i < n; i += NH_T) {
    double s = 0.0;
    for (int j = 0; j < ncol; ++j) s = fma(QH(i, j), gh[j], s);
    g[i] += s;
  }
  double s2 = 0.0;
  for (int i = tid; i < n; i += NH_T) s2 = fma(g[i], g[i], s2);
  s2 = nh_block_sum(s2, sh.red);
  const double gamma = hypot(1.0, sqrt(s2));
  for (int j = k + tid; j < ncol; j += NH_T) AH(n, j) *= gamma;
  nh_sync();
  return gamma;
}

template <int MAXN>
KS_DEVICE void ds_nhep_body(const DSArgs &a, double *smem, int smem_bytes) {
  __shared__ NhShared<MAXN> sh;
  __shared__ double wr[MAXN], wi[MAXN], errs[MAXN];
  __shared__ double hg[MAXN], hgh[MAXN];  // harmonic extraction: g and ghat
  const int tid = nh_tid();
  const int n = a.st ? a.st->m : a.n;
  const int ld = a.ld, l = a.l, flags = a.flags;
  // stage A (rows 0..n) and, when it fits too, Q in shared memory
  const bool sa = smem && nh_smem_a(n) <= (size_t)smem_bytes;
  const bool sq = sa && nh_smem_a(n) + nh_smem_q(n) <= (size_t)smem_bytes;
  double *A = sa ? smem : a.H;
  const int lda = sa ? nh_stride_a(n) : ld;
  double *Q = sq ? smem + (size_t)lda * n : a.Q;
  const int ldq = sq ? nh_stride_q(n) : ld;
  if (sa)
    for (int i = tid; i < (n + 1) * n; i += NH_T) AH(i % (n + 1), i / (n + 1)) = a.H[i % (n + 1) + (size_t)(i / (n + 1)) * ld];
  if (sq && !(flags & DS_DO_SOLVE))
    for (int i = tid; i < n * n; i += NH_T) QH(i % n, i / n) = a.Q[i % n + (size_t)(i / n) * ld];
  if (tid == 0) {
    sh.fail = 0;
    sh.cmd = 0;
  }
  nh_sync();
  const double beta = a.st ? a.st->beta_out : 0.0;
  double hgamma = 1.0;  // correction factor of the residual estimates (1 for Ritz extraction)
  if (flags & DS_DO_SOLVE) {
    // harmonic translation, with the Schur-vector storage as scratch before it is set to the identity
    if (a.harmonic && n > 1) hgamma = nh_harmonic_translate(A, lda, n, a.target, beta, Q, ldq, hg, sh);
    nh_sync();
    for (int i = tid; i < n * n; i += NH_T) QH(i % n, i / n) = ((i % n) == (i / n)) ? 1.0 : 0.0;
    nh_sync();
    if (n > 1 && !sh.fail) {
      if (a.raw || a.harmonic) nh_hessenberg(A, lda, Q, ldq, n, l, sh);
      nh_francis(A, lda, Q, ldq, n, l, sh);
    }
    nh_sync();
  }
  if (tid == 0) nh_eigs(A, lda, n, 0, wr, wi);
  nh_sync();
  if ((flags & DS_DO_SORT) && !sh.fail) {
    int cplx = 0;
    for (int i = l + tid; i + 1 < n; i += NH_T) cplx |= AH(i + 1, i) != 0.0;
    if (!__syncthreads_or(cplx)) {
      nh_sort_real(A, lda, Q, ldq, n, l, a.which, a.target, wr, sh);
    } else {
      // selection sort (DSSort_NHEP_Total), thread 0 chooses, the block moves blocks
      for (int i = l; i < n - 1; ++i) {
        if (tid == 0) {
          double re = wr[i], im = wi[i];
          int pos = 0;
          int j = (im != 0.0) ? i + 2 : i + 1;
          for (; j < n; ++j) {
            if (nh_cmp(a.which, a.target, re, im, wr[j], wi[j]) > 0) { re = wr[j]; im = wi[j]; pos = j; }
            if (wi[j] != 0.0) j++;
          }
          sh.i2 = pos;
        }
        nh_sync();
        const int pos = sh.i2;
        if (pos) {
          if (nh_move(A, lda, Q, ldq, n, pos, i, sh)) {
            if (tid == 0) sh.fail = 2;
            nh_sync();
            break;
          }
          nh_sync();
          if (tid == 0) nh_eigs(A, lda, n, i, wr, wi);
          nh_sync();
        }
        if (wi[i] != 0.0) i++;
      }
    }
  }
  nh_sync();
  if (flags & DS_DO_EXTRAROW) {
    // A(n, :) = Q^T A(n, :)
    double *x = sh.v;
    for (int i = tid; i < n; i += NH_T) x[i] = AH(n, i);
    nh_sync();
    for (int i = tid; i < n; i += NH_T) {
      double s0 = 0.0, s1 = 0.0;
      int j = 0;
      for (; j + 1 < n; j += 2) {
        s0 = fma(QH(j, i), x[j], s0);
        s1 = fma(QH(j + 1, i), x[j + 1], s1);
      }
      if (j < n) s0 = fma(QH(j, i), x[j], s0);
      errs[i] = s0 + s1;
    }
    nh_sync();
    for (int i = tid; i < n; i += NH_T) AH(n, i) = errs[i];
    nh_sync();
  }
  for (int i = tid; i < n; i += NH_T) {
    a.eigr[i] = wr[i];
    if (a.eigi) a.eigi[i] = wi[i];
  }
  if (!(flags & DS_DO_CONTROL)) {
    if (tid == 0 && a.ctl) a.ctl->ds_error = sh.fail;
  } else {
    // residual estimates for k = l..n-1, one eigenvector per thread (DSVectors_NHEP_Eigen_Some): the Ritz vector
    // is Q x with x the eigenvector of the quasi-triangular T, so its norm is ||x|| (Q is orthogonal) and only
    // its last entry Q(n-1, :) x is formed; harmonic extraction scales the estimate by gamma (epskrylov.c:265)
    // max |T(i, j)| over the upper Hessenberg part: columns split over the block, then a max over the warps
    double tnorm = 0.0;
    for (int j = tid; j < n; j += NH_T)
      for (int i = 0; i <= j + 1 && i < n; ++i) tnorm = fmax(tnorm, fabs(AH(i, j)));
    for (int o = 16; o > 0; o >>= 1) tnorm = fmax(tnorm, __shfl_xor_sync(0xffffffffu, tnorm, o));
    if (lane_id() == 0) sh.red[tid >> 5] = tnorm;
    nh_sync();
    tnorm = sh.red[0];
    for (int w = 1; w < NH_T / 32; ++w) tnorm = fmax(tnorm, sh.red[w]);
    double xr[MAXN], xi[MAXN];
    for (int k = l + tid; k < n; k += NH_T) {
      errs[k] = -1.0;
      if (k > 0 && AH(k, k - 1) != 0.0) continue;  // second row of a 2x2 block: handled by the first
      const int cplx = nh_eigvec(A, lda, n, k, tnorm, xr, xi);
      double yl_r = 0.0, yl_i = 0.0, nr2 = 0.0, ni2 = 0.0;
      for (int j = 0; j <= k + cplx; ++j) {
        yl_r = fma(QH(n - 1, j), xr[j], yl_r);
        nr2 = fma(xr[j], xr[j], nr2);
        if (cplx) {
          yl_i = fma(QH(n - 1, j), xi[j], yl_i);
          ni2 = fma(xi[j], xi[j], ni2);
        }
      }
      const double nrm = sqrt(nr2 + ni2);
      const double rn = (cplx ? hypot(yl_r, yl_i) : fabs(yl_r)) / nrm * (beta * hgamma);
      const double w = hypot(wr[k], wi[k]);
      errs[k] = ds_conv_errest(a, rn, w);
      if (cplx) errs[k + 1] = errs[k];
    }
    nh_sync();
    // convergence marker, restart sizes and stopping test (thread 0), then the harmonic recovery (block)
    if (tid == 0) {
      int kk;
      for (kk = l; kk < n; ++kk) {
        a.errest[kk] = errs[kk];
        if (errs[kk] >= a.tol) break;
        if (wi[kk] != 0.0 && kk + 1 < n) {
          a.errest[kk + 1] = errs[kk];
          kk++;
        }
      }
      int reason = 0;
      if (kk >= a.nev) reason = 1;
      else if (a.its >= a.max_it) reason = -1;
      const int breakdown = a.st ? a.st->breakdown : 0;
      int lkeep;
      if (reason != 0 || breakdown || kk == n) lkeep = 0;
      else {
        lkeep = (int)((n - kk) * a.keep);
        if (lkeep < 1) lkeep = 1;
        // DSGetTruncateSize_Default: do not split a 2x2 block
        if (AH(kk + lkeep, kk + lkeep - 1) != 0.0) {
          if (kk + lkeep < n - 1) lkeep++;
          else lkeep--;
        }
      }
      if (!a.lock && lkeep > 0) { lkeep += kk; kk = 0; }
      sh.i0 = kk;
      sh.i1 = lkeep;
      sh.i3 = reason;
      sh.cmd = (reason == 0 && !(breakdown || kk == n)) ? 1 : 0;  // restart with truncation
      sh.G[0] = 1.0;
    }
    nh_sync();
    if (a.harmonic && sh.cmd && !sh.fail) {
      const double g2 = nh_harmonic_recover(A, lda, Q, ldq, n, sh.i0, sh.i1, beta, hg, hgh, sh);
      for (int i = tid; i < n; i += NH_T) a.work[i] = hg[i];  // g~ for the residual-vector update
      if (tid == 0) sh.G[0] = g2;
      nh_sync();
    }
    if (tid == 0) {
      const int kk = sh.i0, lkeep = sh.i1, reason = sh.i3;
      const int breakdown = a.st ? a.st->breakdown : 0;
      KSControl *ctl = a.ctl;
      if (sh.cmd) {
        // DSTruncate_NHEP: move the extra row to row kk+lkeep
        const int nn = kk + lkeep;
        for (int i = l; i < nn; ++i) AH(nn, i) = AH(n, i);
        for (int i = l; i < n; ++i) AH(n, i) = 0.0;
      }
      ctl->nconv = kk;
      ctl->l = lkeep;
      ctl->reason = reason;
      ctl->nv = n;
      ctl->breakdown = breakdown;
      ctl->need_start = (reason == 0 && (breakdown || kk == n) && kk < a.nev) ? 1 : 0;
      ctl->ds_error = sh.fail;
      ctl->beta = beta;
      ctl->hgamma = sh.G[0];
    }
  }
  nh_sync();
  if (sa)
    for (int i = tid; i < (n + 1) * n; i += NH_T) a.H[i % (n + 1) + (size_t)(i / (n + 1)) * ld] = AH(i % (n + 1), i / (n + 1));
  if (sq)
    for (int i = tid; i < n * n; i += NH_T) a.Q[i % n + (size_t)(i / n) * ld] = QH(i % n, i / n);
  nh_sync();
}

__global__ void __launch_bounds__(NH_T) k_ds_nhep(DSArgs a, int smem_bytes) {
  extern __shared__ double nh_dyn[];
  ds_nhep_body<NH_MAXN>(a, nh_dyn, smem_bytes);
}

// projected problems above 144 rows: A and Q transformed in place in the caller's arrays
__global__ void __launch_bounds__(NH_T) k_ds_nhep_wide(DSArgs a) { ds_nhep_body<NH_WIDE_MAXN>(a, nullptr, 0); }

// one block per non-symmetric instance of a batch (grid-stride over the live list)
__global__ void __launch_bounds__(NH_T) k_batch_ds_nhep(const BatchInst *I, const int *list, const BatchHdr *h,
                                                         int smem_bytes) {
  extern __shared__ double nh_dyn[];
  for (int v = blockIdx.x; v < h->n_inst; v += gridDim.x) {
    const BatchInst &p = I[list[v]];
    if (p.phase != BP_ITER || p.hermitian) continue;
    nh_sync();
    ds_nhep_body<NH_MAXN>(batch_ds_args(p), nh_dyn, smem_bytes);
  }
}

// eigenvectors of the leading n x n quasi-triangular block, normalised (DSVectors_NHEP_Eigen_All with back = "A")
template <int MAXN>
__global__ void __launch_bounds__(32) k_nhep_vectors(const double *A, int lda, int n, double *X) {
  const int lane = lane_id();
  double tnorm = 0.0;
  for (int j = 0; j < n; ++j)
    for (int i = 0; i <= j + 1 && i < n; ++i) tnorm = fmax(tnorm, fabs(AH(i, j)));
  double xr[MAXN], xi[MAXN];
  for (int k = lane; k < n; k += 32) {
    if (k > 0 && AH(k, k - 1) != 0.0) continue;
    const int cplx = nh_eigvec(A, lda, n, k, tnorm, xr, xi);
    double s = 0.0;
    for (int i = 0; i < n; ++i) s += xr[i] * xr[i] + xi[i] * xi[i];
    const double inv = 1.0 / sqrt(s);
    for (int i = 0; i < n; ++i) {
      X[i + (size_t)k * lda] = xr[i] * inv;
      if (cplx) X[i + (size_t)(k + 1) * lda] = xi[i] * inv;
    }
  }
}

// dynamic shared memory of each solver kernel: at most NH_SMEM_MAX, and what the device's opt-in limit leaves
// beside the kernel's own static shared memory (set once, before any launch is captured into a graph)
static int g_nh_dyn[2] = {-1, -1};  // k_ds_nhep, k_batch_ds_nhep

template <typename K>
static cudaError_t nh_allow_smem(K kernel, int *dyn) {
  int dev = 0, optin = 0;
  cudaFuncAttributes fa;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, kernel);
  if (e != cudaSuccess) return e;
  const int room = optin - (int)fa.sharedSizeBytes;
  *dyn = room < NH_SMEM_MAX ? (room > 0 ? room : 0) : NH_SMEM_MAX;
  return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, *dyn);
}

// dynamic shared memory for problems of size up to n_max: A, and Q when both fit in the kernel's allowance
static int nh_smem_bytes(int n_max, int allowed) {
  size_t b = nh_smem_a(n_max);
  if (b + nh_smem_q(n_max) <= (size_t)allowed) b += nh_smem_q(n_max);
  return b <= (size_t)allowed ? (int)b : 0;
}

cudaError_t prepare_ds_nhep() {
  static cudaError_t attr = [] {
    cudaError_t e = nh_allow_smem(k_ds_nhep, &g_nh_dyn[0]);
    return e != cudaSuccess ? e : nh_allow_smem(k_batch_ds_nhep, &g_nh_dyn[1]);
  }();
  return attr;
}

int ds_nhep_max_n() { return NH_WIDE_MAXN; }

cudaError_t launch_ds_nhep(const DSArgs &a, int n_max, cudaStream_t s) {
  if (n_max > NH_WIDE_MAXN || a.ld < n_max) return cudaErrorInvalidValue;
  if (n_max > NH_MAXN) {
    k_ds_nhep_wide<<<1, NH_T, 0, s>>>(a);
    return cudaGetLastError();
  }
  const cudaError_t attr = prepare_ds_nhep();
  if (attr != cudaSuccess) return attr;
  const int bytes = nh_smem_bytes(n_max, g_nh_dyn[0]);
  k_ds_nhep<<<1, NH_T, bytes, s>>>(a, bytes);
  return cudaGetLastError();
}

cudaError_t launch_batch_ds_nhep(const BatchInst *I, const int *list, const BatchHdr *h, int grid, int max_ld,
                                 cudaStream_t s) {
  if (max_ld > NH_MAXN) return cudaErrorInvalidValue;
  const cudaError_t attr = prepare_ds_nhep();
  if (attr != cudaSuccess) return attr;
  const int bytes = nh_smem_bytes(max_ld, g_nh_dyn[1]);
  k_batch_ds_nhep<<<grid, NH_T, bytes, s>>>(I, list, h, bytes);
  return cudaGetLastError();
}

cudaError_t launch_nhep_vectors(double *T, int ld, int n, double *X, cudaStream_t s) {
  if (n > NH_WIDE_MAXN) return cudaErrorInvalidValue;
  if (n > NH_MAXN) k_nhep_vectors<NH_WIDE_MAXN><<<1, 32, 0, s>>>(T, ld, n, X);
  else k_nhep_vectors<NH_MAXN><<<1, 32, 0, s>>>(T, ld, n, X);
  return cudaGetLastError();
}

#undef AH
#undef QH

}  // namespace ksg
