// k_ds_nhep.cu -- projected problem of the non-symmetric Krylov-Schur iteration, solved on the device in FP64.
//
// One warp per projected problem (lane 0 runs the scalar recurrences, all lanes apply the transformations), so
// the same code serves the single large solve and, later, many small solves side by side.  It follows the
// reference's DSNHEP path:
//   DSSolve_NHEP_Private (src/sys/classes/ds/impls/dsutil.c:21-87): Householder reduction to Hessenberg form of the
//     rows/columns from l on (gehrd with ILO = l+1) when the matrix holds the Krylov-Schur form, then the real
//     Schur form by Francis double-shift QR (the algorithm of hseqr/lahqr) with standardised 2x2 blocks (lanv2);
//   DSSort_NHEP_Total (dsutil.c:93-171): selection sort by the criterion, moving blocks by direct swapping of
//     adjacent Schur blocks (Bai and Demmel 1993, the algorithm of trexc/laexc);
//   DSUpdateExtraRow_NHEP (dsnhep.c:318-340), DSVectors_NHEP_Eigen_Some (dsnhep.c:101-166) for the residual
//     estimates of EPSKrylovConvergence (epskrylov.c:207-295), DSGetTruncateSize (dsops.c:329-344) and
//     DSTruncate_NHEP (dsnhep.c:394-425).
// A and Q stay in global memory (they are at most 144 x 144 and L1/L2 resident).
#include <float.h>

#include "batch_types.h"
#include "common.cuh"
#include "kernels.h"
#include "ks_types.h"

namespace ksg {

constexpr int NH_MAXN = 144;

#define AH(i, j) A[(i) + (size_t)(j) * ld]
#define QH(i, j) Q[(i) + (size_t)(j) * ld]

struct NhShared {
  double v[NH_MAXN + 4];
  double G[16];
  double tau, beta, cs, sn;
  int cmd, i0, i1, i2, i3;
  int fail;
};

KS_DEVICE int lane_id() { return threadIdx.x & 31; }

// Householder vector of x[0..m-1] (lane 0): x becomes v with v[0] = 1; returns tau, *beta = resulting head
__device__ double nh_house(int m, double *x, double *beta) {
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

// warp-parallel reflector applications (v, tau in shared memory)
__device__ void nh_refl_left(double *A, int ld, int r0, int m, int c0, int c1, const double *v, double tau) {
  for (int j = c0 + lane_id(); j <= c1; j += 32) {
    double s = 0.0;
    for (int i = 0; i < m; ++i) s = fma(v[i], AH(r0 + i, j), s);
    s *= tau;
    for (int i = 0; i < m; ++i) AH(r0 + i, j) -= s * v[i];
  }
}
__device__ void nh_refl_right(double *A, int ld, int c0, int m, int r0, int r1, const double *v, double tau) {
  for (int i = r0 + lane_id(); i <= r1; i += 32) {
    double s = 0.0;
    for (int j = 0; j < m; ++j) s = fma(AH(i, c0 + j), v[j], s);
    s *= tau;
    for (int j = 0; j < m; ++j) AH(i, c0 + j) -= s * v[j];
  }
}
// BLAS rot on rows (x: row p, y: row p+1, columns c0..c1) or columns (rows r0..r1)
__device__ void nh_rot_rows(double *A, int ld, int p, int c0, int c1, double c, double s) {
  for (int j = c0 + lane_id(); j <= c1; j += 32) {
    const double x = AH(p, j), y = AH(p + 1, j);
    AH(p, j) = c * x + s * y;
    AH(p + 1, j) = c * y - s * x;
  }
}
__device__ void nh_rot_cols(double *A, int ld, int p, int r0, int r1, double c, double s) {
  for (int i = r0 + lane_id(); i <= r1; i += 32) {
    const double x = AH(i, p), y = AH(i, p + 1);
    AH(i, p) = c * x + s * y;
    AH(i, p + 1) = c * y - s * x;
  }
}

// 2x2 standardisation (lane 0): [a b; c d] -> G^T [a b; c d] G, G = [cs -sn; sn cs]
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

// standardise the 2x2 block at (i, i+1) and propagate to T and Q (whole warp)
__device__ void nh_std_block(double *A, double *Q, int ld, int n, int i, NhShared &sh) {
  if (lane_id() == 0) {
    double a = AH(i, i), b = AH(i, i + 1), c = AH(i + 1, i), d = AH(i + 1, i + 1), cs, sn;
    nh_std2x2(a, b, c, d, cs, sn);
    AH(i, i) = a; AH(i, i + 1) = b; AH(i + 1, i) = c; AH(i + 1, i + 1) = d;
    sh.cs = cs;
    sh.sn = sn;
  }
  __syncwarp();
  const double cs = sh.cs, sn = sh.sn;
  if (i + 2 < n) nh_rot_rows(A, ld, i, i + 2, n - 1, cs, sn);
  if (i > 0) nh_rot_cols(A, ld, i, 0, i - 1, cs, sn);
  nh_rot_cols(Q, ld, i, 0, n - 1, cs, sn);
  __syncwarp();
}

// Hessenberg reduction from column ilo (rows/columns before ilo already triangular), accumulated into Q
__device__ void nh_hessenberg(double *A, double *Q, int ld, int n, int ilo, NhShared &sh) {
  for (int c = ilo; c < n - 2; ++c) {
    const int m = n - c - 1;
    if (lane_id() == 0) {
      for (int i = 0; i < m; ++i) sh.v[i] = AH(c + 1 + i, c);
      double beta;
      sh.tau = nh_house(m, sh.v, &beta);
      sh.beta = beta;
    }
    __syncwarp();
    const double tau = sh.tau;
    if (tau != 0.0) {
      nh_refl_left(A, ld, c + 1, m, c, n - 1, sh.v, tau);
      __syncwarp();
      nh_refl_right(A, ld, c + 1, m, 0, n - 1, sh.v, tau);
      nh_refl_right(Q, ld, c + 1, m, 0, n - 1, sh.v, tau);
      __syncwarp();
      if (lane_id() == 0) {
        AH(c + 1, c) = sh.beta;
        for (int i = 1; i < m; ++i) AH(c + 1 + i, c) = 0.0;
      }
    }
    __syncwarp();
  }
}

// real Schur form of the Hessenberg matrix (rows/columns before ilo triangular); returns 0 or 1 (no convergence)
__device__ int nh_francis(double *A, double *Q, int ld, int n, int ilo, NhShared &sh) {
  const double eps = DBL_EPSILON;
  const double smlnum = DBL_MIN * ((double)n / eps);
  for (int i = ilo + 2 + lane_id(); i < n; i += 32)
    for (int j = ilo; j < i - 1; ++j) AH(i, j) = 0.0;
  __syncwarp();
  int ihi = n - 1, its = 0, totits = 0;
  const int maxtot = 40 * (n > 10 ? n : 10);
  for (;;) {
    // lane 0 decides: cmd 0 done, 1 standardise block at i0, 2 Francis sweep on [i0, i1]
    if (lane_id() == 0) {
      sh.cmd = 0;
      while (ihi >= ilo) {
        int l;
        for (l = ihi; l > ilo; --l) {
          const double hll = fabs(AH(l, l - 1));
          if (hll <= smlnum) break;
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
            if (ba * (ab / s) <= fmax(smlnum, eps * (bb * (aa / s)))) break;
          }
        }
        if (l > ilo) AH(l, l - 1) = 0.0;
        if (l >= ihi) {
          ihi -= 1;
          its = 0;
          continue;
        }
        if (l == ihi - 1) {
          sh.cmd = 1;
          sh.i0 = l;
          ihi -= 2;
          its = 0;
          break;
        }
        if (++totits > maxtot) {
          sh.fail = 1;
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
        double v0 = h21s * AH(m, m + 1) + (AH(m, m) - rt1r) * ((AH(m, m) - rt2r) / sc) - rt1i * (rt2i / sc);
        double v1 = h21s * (AH(m, m) + AH(m + 1, m + 1) - rt1r - rt2r);
        double v2 = h21s * AH(m + 2, m + 1);
        sc = fabs(v0) + fabs(v1) + fabs(v2);
        sh.v[0] = v0 / sc;
        sh.v[1] = v1 / sc;
        sh.v[2] = v2 / sc;
        sh.cmd = 2;
        sh.i0 = m;
        sh.i1 = ihi;
        break;
      }
    }
    __syncwarp();
    const int cmd = sh.cmd;
    if (cmd == 0) break;
    if (cmd == 1) {
      nh_std_block(A, Q, ld, n, sh.i0, sh);
      continue;
    }
    // bulge chase over [m, hi]
    const int m = sh.i0, hi = sh.i1;
    for (int k = m; k <= hi - 1; ++k) {
      const int nr = (3 < hi - k + 1) ? 3 : hi - k + 1;
      if (lane_id() == 0) {
        if (k > m)
          for (int i = 0; i < nr; ++i) sh.v[i] = AH(k + i, k - 1);
        double beta;
        sh.tau = nh_house(nr, sh.v, &beta);
        if (k > m) {
          AH(k, k - 1) = beta;
          AH(k + 1, k - 1) = 0.0;
          if (k < hi - 1) AH(k + 2, k - 1) = 0.0;
        }
      }
      __syncwarp();
      const double tau = sh.tau;
      if (tau != 0.0) {
        nh_refl_left(A, ld, k, nr, k, n - 1, sh.v, tau);
        __syncwarp();
        const int r1 = (k + 3 < hi) ? k + 3 : hi;
        nh_refl_right(A, ld, k, nr, 0, r1, sh.v, tau);
        nh_refl_right(Q, ld, k, nr, 0, n - 1, sh.v, tau);
      }
      __syncwarp();
    }
  }
  return sh.fail;
}

// small Sylvester solve T11 X - X T22 = B (Kronecker system, complete pivoting), lane 0
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
__device__ int nh_swap(double *A, double *Q, int ld, int n, int j1, int n1, int n2, NhShared &sh) {
  const int m = n1 + n2;
  if (n1 == 1 && n2 == 1) {
    const int j2 = j1 + 1;
    if (lane_id() == 0) {
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
    __syncwarp();
    const double c = sh.cs, s = sh.sn;
    if (j2 + 1 < n) nh_rot_rows(A, ld, j1, j2 + 1, n - 1, c, s);
    if (j1 > 0) nh_rot_cols(A, ld, j1, 0, j1 - 1, c, s);
    nh_rot_cols(Q, ld, j1, 0, n - 1, c, s);
    __syncwarp();
    if (lane_id() == 0) {
      AH(j1, j1) = sh.G[1];
      AH(j2, j2) = sh.G[0];
    }
    __syncwarp();
    return 0;
  }
  if (lane_id() == 0) {
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
  __syncwarp();
  if (sh.cmd) return 1;
  const double *G = sh.G;
  // left: rows j1..j1+m-1 over columns j1..n-1
  for (int j = j1 + lane_id(); j < n; j += 32) {
    double t[4];
    for (int i = 0; i < m; ++i) {
      double s = 0.0;
      for (int k = 0; k < m; ++k) s += G[k + i * 4] * AH(j1 + k, j);
      t[i] = s;
    }
    for (int i = 0; i < m; ++i) AH(j1 + i, j) = t[i];
  }
  __syncwarp();
  // right: columns j1..j1+m-1 over rows 0..j1+m-1; Q over all rows
  for (int i = lane_id(); i < j1 + m; i += 32) {
    double t[4];
    for (int j = 0; j < m; ++j) {
      double s = 0.0;
      for (int k = 0; k < m; ++k) s += AH(i, j1 + k) * G[k + j * 4];
      t[j] = s;
    }
    for (int j = 0; j < m; ++j) AH(i, j1 + j) = t[j];
  }
  for (int i = lane_id(); i < n; i += 32) {
    double t[4];
    for (int j = 0; j < m; ++j) {
      double s = 0.0;
      for (int k = 0; k < m; ++k) s += QH(i, j1 + k) * G[k + j * 4];
      t[j] = s;
    }
    for (int j = 0; j < m; ++j) QH(i, j1 + j) = t[j];
  }
  __syncwarp();
  if (lane_id() == 0)
    for (int i = n2; i < m; ++i)
      for (int j = 0; j < n2; ++j) AH(j1 + i, j1 + j) = 0.0;
  __syncwarp();
  if (n2 == 2) nh_std_block(A, Q, ld, n, j1, sh);
  else {
    if (lane_id() == 0) AH(j1 + 1, j1) = 0.0;
    __syncwarp();
  }
  if (n1 == 2) nh_std_block(A, Q, ld, n, j1 + n2, sh);
  return 0;
}

// move the block at ifst up to ilst (ifst > ilst); 0 or 1 (rejected swap)
__device__ int nh_move(double *A, double *Q, int ld, int n, int ifst, int ilst, NhShared &sh) {
  if (ifst > 0 && AH(ifst, ifst - 1) != 0.0) ifst--;
  int nbf = (ifst < n - 1 && AH(ifst + 1, ifst) != 0.0) ? 2 : 1;
  if (ilst > 0 && AH(ilst, ilst - 1) != 0.0) ilst--;
  int here = ifst;
  while (here > ilst) {
    const int nbnext = (here >= 2 && AH(here - 1, here - 2) != 0.0) ? 2 : 1;
    if (nh_swap(A, Q, ld, n, here - nbnext, nbnext, nbf, sh)) return 1;
    __syncwarp();
    if (nbf == 2 && AH(here - nbnext + 1, here - nbnext) == 0.0) nbf = 1;
    here -= nbnext;
  }
  return 0;
}

__device__ void nh_eigs(const double *A, int ld, int n, int from, double *wr, double *wi) {
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
__device__ int nh_eigvec(const double *A, int ld, int n, int k, double tnorm, double *xr, double *xi) {
  const double eps = DBL_EPSILON;
  const double smin = fmax(eps * tnorm, DBL_MIN / eps);
  for (int i = 0; i < n; ++i) { xr[i] = 0.0; xi[i] = 0.0; }
  const int cplx = (k < n - 1 && AH(k + 1, k) != 0.0);
  if (!cplx) {
    const double lam = AH(k, k);
    xr[k] = 1.0;
    for (int i = k - 1; i >= 0; --i) {
      if (i > 0 && AH(i, i - 1) != 0.0) {
        double r0 = 0.0, r1 = 0.0;
        for (int j = i + 1; j <= k; ++j) { r0 -= AH(i - 1, j) * xr[j]; r1 -= AH(i, j) * xr[j]; }
        const double a = AH(i - 1, i - 1) - lam, b = AH(i - 1, i), c = AH(i, i - 1), d = AH(i, i) - lam;
        double det = a * d - b * c;
        if (fabs(det) < smin) det = copysign(smin, det);
        xr[i - 1] = (r0 * d - b * r1) / det;
        xr[i] = (a * r1 - c * r0) / det;
        i--;
      } else {
        double s = 0.0;
        for (int j = i + 1; j <= k; ++j) s -= AH(i, j) * xr[j];
        double den = AH(i, i) - lam;
        if (fabs(den) < smin) den = smin;
        xr[i] = s / den;
      }
      double mx = 0.0;
      for (int j = i; j <= k; ++j) mx = fmax(mx, fabs(xr[j]));
      if (mx > 1e150)
        for (int j = 0; j <= k; ++j) xr[j] /= mx;
    }
    return 0;
  }
  const int ki = k + 1;
  const double wr = AH(k, k);
  const double wim = sqrt(fabs(AH(k, ki))) * sqrt(fabs(AH(ki, k)));
  if (fabs(AH(k, ki)) >= fabs(AH(ki, k))) { xr[k] = 1.0; xi[ki] = wim / AH(k, ki); }
  else { xr[k] = -wim / AH(ki, k); xi[ki] = 1.0; }
  for (int i = k - 1; i >= 0; --i) {
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
    } else {
      double sr = 0.0, si = 0.0;
      for (int j = i + 1; j <= ki; ++j) { sr -= AH(i, j) * xr[j]; si -= AH(i, j) * xi[j]; }
      double denr = AH(i, i) - wr, deni = -wim;
      double dd = denr * denr + deni * deni;
      if (dd < smin * smin) { denr = smin; deni = 0.0; dd = smin * smin; }
      xr[i] = (sr * denr + si * deni) / dd;
      xi[i] = (si * denr - sr * deni) / dd;
    }
    double mx = 0.0;
    for (int j = i; j <= ki; ++j) mx = fmax(mx, fabs(xr[j]) + fabs(xi[j]));
    if (mx > 1e150)
      for (int j = 0; j <= ki; ++j) { xr[j] /= mx; xi[j] /= mx; }
  }
  return 1;
}

KS_DEVICE void ds_nhep_body(const DSArgs &a) {
  __shared__ NhShared sh;
  __shared__ double wr[NH_MAXN], wi[NH_MAXN], errs[NH_MAXN];
  const int lane = lane_id();
  const int n = a.st ? a.st->m : a.n;
  const int ld = a.ld, l = a.l, flags = a.flags;
  double *A = a.H, *Q = a.Q;
  if (lane == 0) {
    sh.fail = 0;
    sh.cmd = 0;
  }
  __syncwarp();
  if (flags & DS_DO_SOLVE) {
    for (int i = lane; i < n * n; i += 32) QH(i % n, i / n) = ((i % n) == (i / n)) ? 1.0 : 0.0;
    __syncwarp();
    if (n > 1) {
      if (a.raw) nh_hessenberg(A, Q, ld, n, l, sh);
      nh_francis(A, Q, ld, n, l, sh);
    }
    __syncwarp();
  }
  if (lane == 0) nh_eigs(A, ld, n, 0, wr, wi);
  __syncwarp();
  if ((flags & DS_DO_SORT) && !sh.fail) {
    // selection sort (DSSort_NHEP_Total), lane 0 chooses, the warp moves blocks
    for (int i = l; i < n - 1; ++i) {
      if (lane == 0) {
        double re = wr[i], im = wi[i];
        int pos = 0;
        int j = (im != 0.0) ? i + 2 : i + 1;
        for (; j < n; ++j) {
          int res;
          {
            double av, bv;
            switch (a.which) {
              case 1: av = hypot(re, im); bv = hypot(wr[j], wi[j]); res = av < bv ? 1 : (av > bv ? -1 : 0); break;
              case 2: av = hypot(re, im); bv = hypot(wr[j], wi[j]); res = av > bv ? 1 : (av < bv ? -1 : 0); break;
              case 3: res = re < wr[j] ? 1 : (re > wr[j] ? -1 : 0); break;
              case 4: res = re > wr[j] ? 1 : (re < wr[j] ? -1 : 0); break;
              case 5: av = fabs(im); bv = fabs(wi[j]); res = av < bv ? 1 : (av > bv ? -1 : 0); break;
              case 6: av = fabs(im); bv = fabs(wi[j]); res = av > bv ? 1 : (av < bv ? -1 : 0); break;
              default: res = 0;
            }
          }
          if (res > 0) { re = wr[j]; im = wi[j]; pos = j; }
          if (wi[j] != 0.0) j++;
        }
        sh.i2 = pos;
      }
      __syncwarp();
      const int pos = sh.i2;
      if (pos) {
        if (nh_move(A, Q, ld, n, pos, i, sh)) {
          if (lane == 0) sh.fail = 2;
          __syncwarp();
          break;
        }
        __syncwarp();
        if (lane == 0) nh_eigs(A, ld, n, i, wr, wi);
        __syncwarp();
      }
      if (wi[i] != 0.0) i++;
    }
  }
  __syncwarp();
  if (flags & DS_DO_EXTRAROW) {
    // A(n, :) = Q^T A(n, :)
    double *x = sh.v;
    for (int i = lane; i < n; i += 32) x[i] = AH(n, i);
    __syncwarp();
    for (int i = lane; i < n; i += 32) {
      double s = 0.0;
      for (int j = 0; j < n; ++j) s = fma(QH(j, i), x[j], s);
      errs[i] = s;
    }
    __syncwarp();
    for (int i = lane; i < n; i += 32) AH(n, i) = errs[i];
    __syncwarp();
  }
  for (int i = lane; i < n; i += 32) {
    a.eigr[i] = wr[i];
    if (a.eigi) a.eigi[i] = wi[i];
  }
  if (!(flags & DS_DO_CONTROL)) {
    if (lane == 0 && a.ctl) a.ctl->ds_error = sh.fail;
    return;
  }
  // residual estimates for k = l..n-1, one eigenvector per lane (DSVectors_NHEP_Eigen_Some)
  const double beta = a.st ? a.st->beta_out : 0.0;
  double tnorm = 0.0;
  for (int j = 0; j < n; ++j)
    for (int i = 0; i <= j + 1 && i < n; ++i) tnorm = fmax(tnorm, fabs(AH(i, j)));
  double xr[NH_MAXN], xi[NH_MAXN];
  for (int k = l + lane; k < n; k += 32) {
    errs[k] = -1.0;
    if (k > 0 && AH(k, k - 1) != 0.0) continue;  // second row of a 2x2 block: handled by the first
    const int cplx = nh_eigvec(A, ld, n, k, tnorm, xr, xi);
    double yl_r = 0.0, yl_i = 0.0, nr2 = 0.0, ni2 = 0.0;
    for (int i = 0; i < n; ++i) {
      double sr = 0.0, si = 0.0;
      for (int j = 0; j <= k + cplx; ++j) {
        sr = fma(QH(i, j), xr[j], sr);
        if (cplx) si = fma(QH(i, j), xi[j], si);
      }
      nr2 += sr * sr;
      ni2 += si * si;
      if (i == n - 1) { yl_r = sr; yl_i = si; }
    }
    const double nrm = sqrt(nr2 + ni2);
    const double rn = (cplx ? hypot(yl_r, yl_i) : fabs(yl_r)) / nrm * beta;
    const double w = hypot(wr[k], wi[k]);
    errs[k] = (w != 0.0) ? rn / w : DBL_MAX;
    if (cplx) errs[k + 1] = errs[k];
  }
  __syncwarp();
  if (lane == 0) {
    int kk;
    for (kk = l; kk < n; ++kk) {
      a.errest[kk] = errs[kk];
      if (errs[kk] >= a.tol) break;
      if (wi[kk] != 0.0 && kk + 1 < n) {
        a.errest[kk + 1] = errs[kk];
        kk++;
      }
    }
    KSControl *ctl = a.ctl;
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
    if (reason == 0 && !(breakdown || kk == n)) {
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
  }
}

__global__ void __launch_bounds__(32) k_ds_nhep(DSArgs a) { ds_nhep_body(a); }

// one warp per non-symmetric instance of a batch (grid-stride over the live list)
__global__ void __launch_bounds__(32) k_batch_ds_nhep(const BatchInst *I, const int *list, const BatchHdr *h) {
  for (int v = blockIdx.x; v < h->n_inst; v += gridDim.x) {
    const BatchInst &p = I[list[v]];
    if (p.phase != BP_ITER || p.hermitian) continue;
    __syncwarp();
    ds_nhep_body(batch_ds_args(p));
  }
}

// eigenvectors of the leading n x n quasi-triangular block, normalised (DSVectors_NHEP_Eigen_All with back = "A")
__global__ void __launch_bounds__(32) k_nhep_vectors(const double *A, int ld, int n, double *X) {
  const int lane = lane_id();
  double tnorm = 0.0;
  for (int j = 0; j < n; ++j)
    for (int i = 0; i <= j + 1 && i < n; ++i) tnorm = fmax(tnorm, fabs(AH(i, j)));
  double xr[NH_MAXN], xi[NH_MAXN];
  for (int k = lane; k < n; k += 32) {
    if (k > 0 && AH(k, k - 1) != 0.0) continue;
    const int cplx = nh_eigvec(A, ld, n, k, tnorm, xr, xi);
    double s = 0.0;
    for (int i = 0; i < n; ++i) s += xr[i] * xr[i] + xi[i] * xi[i];
    const double inv = 1.0 / sqrt(s);
    for (int i = 0; i < n; ++i) {
      X[i + (size_t)k * ld] = xr[i] * inv;
      if (cplx) X[i + (size_t)(k + 1) * ld] = xi[i] * inv;
    }
  }
}

cudaError_t launch_ds_nhep(const DSArgs &a, int n_max, cudaStream_t s) {
  if (n_max > NH_MAXN) return cudaErrorInvalidValue;
  k_ds_nhep<<<1, 32, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_batch_ds_nhep(const BatchInst *I, const int *list, const BatchHdr *h, int grid, int max_ld,
                                 cudaStream_t s) {
  if (max_ld > NH_MAXN) return cudaErrorInvalidValue;
  k_batch_ds_nhep<<<grid, 32, 0, s>>>(I, list, h);
  return cudaGetLastError();
}

cudaError_t launch_nhep_vectors(double *T, int ld, int n, double *X, cudaStream_t s) {
  if (n > NH_MAXN) return cudaErrorInvalidValue;
  k_nhep_vectors<<<1, 32, 0, s>>>(T, ld, n, X);
  return cudaGetLastError();
}

#undef AH
#undef QH

}  // namespace ksg
