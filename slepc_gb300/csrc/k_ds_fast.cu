// k_ds_fast.cu -- the symmetric projected problem of the Krylov-Schur iteration, solved in mixed precision.
//
// On GB300 a dependent FP64 operation costs 64 cycles, a square root about 690 and a division about 440, so the
// one-thread Givens chains of an FP64 QL solver dominate a restart.  This solver runs those chains in FP32 and
// recovers FP64 accuracy with GPU-wide FP64 matrix products:
//
//   1. k_dsf_eig32: the arrowhead-to-tridiagonal Givens reduction and implicit QL of the reference's DSSolve_HEP_QR
//      (src/sys/classes/ds/impls/hep/dshep.c:221-262, 383-426) in FP32 on the active block [l, n), giving X0.
//   2. four refinement steps of Ogita and Aishima ("Iterative refinement for symmetric eigenvalue decomposition",
//      Japan J. Indust. Appl. Math. 35 (2018) 1007-1035), FP64:
//        P = T X,  S = X^T P,  G = X^T X,  lambda_i = s_ii / g_ii,
//        delta = 2 (||S - diag(lambda)||_F + ||T||_F ||I - G||_F),
//        E_ij = (s_ij + lambda_j r_ij) / (lambda_j - lambda_i) if |lambda_j - lambda_i| > max(delta, tau), else r_ij/2,
//        X <- X + X E   (r = I - G).
//      Eigenvalues closer than tau = 1e-5 * max|lambda| form clusters; the cluster block of S is diagonalised by
//      FP64 Jacobi and X rotated inside the cluster before the update, so no close pair is corrected to first
//      order.  Each step squares the eigenvector error (the 2x2 analysis gives theta -> O(theta^2) independent of
//      the gap); the gap only bounds the FP64 floor u ||T|| / gap, the same as for any backward-stable solver.
//   3. a final cluster pass, one Newton-Schulz step X (3I - X^T X) / 2 that makes X orthogonal to rounding, and the
//      sort by criterion, extra row, convergence test and restart control (k_dsf_finish, the same contract as the
//      FP64 kernel in k_ds_hep.cu).
//   4. an accuracy check before the final cluster pass: outside the clusters every off-diagonal entry of X^T T X must
//      be at rounding level of ||T||, and X^T X at rounding level of I.  Pairs whose gap is just above the cluster
//      threshold can stay mixed after the refinement steps (measured on the 128^3 Laplacian: pairs 1.7e-4 apart at
//      |lambda| ~ 12 left residuals of 1e-7); when the check fails, the FP64 QR solver of k_ds_hep.cu solves the
//      projected problem again from the untouched compact form, so every restart gets FP64-accurate Ritz pairs.
#include <float.h>

#include "common.cuh"
#include "kernels.h"
#include "ks_types.h"

namespace ksg {

constexpr int DSF_THREADS = 256;
constexpr int DSF_MAXN = 144;
constexpr int DSF_CL = 16;     // largest cluster diagonalised as one block (longer runs are split)
constexpr int DSF_TILE = 16;   // output tile of the small FP64 products
constexpr int DSF_ITERS = 4;   // refinement steps
constexpr double DSF_TAU = 1e-5;
// accuracy check before the final cluster pass: |s_ij| <= 256 eps ||T||_F outside clusters; |G - I| <= 1e-12 (the
// refinement's own rounding floor for X^T X is near 2e-13 at ld = 129; the Newton-Schulz step that follows the
// check takes the orthogonality error of X from there to rounding level)
constexpr double DSF_CHECK = 256.0;
constexpr double DSF_CHECK_G = 1e-12;

size_t ds_fast_scratch_doubles(int ld) {
  const int nt = (ld + DSF_TILE - 1) / DSF_TILE;
  return (size_t)5 * ld * ld + (size_t)2 * ld * DSF_CL + ld + 2 * (size_t)nt * nt + 8;
}

DSFArgs ds_fast_layout(double *scratch, int ld) {
  DSFArgs f = {};
  const size_t sq = (size_t)ld * ld;
  const int nt = (ld + DSF_TILE - 1) / DSF_TILE;
  f.ld = ld;
  f.T = scratch;
  f.X = scratch + sq;
  f.P = scratch + 2 * sq;
  f.S = scratch + 3 * sq;
  f.G = scratch + 4 * sq;
  f.W = scratch + 5 * sq;
  f.lam = f.W + (size_t)2 * ld * DSF_CL;
  f.part = f.lam + ld;
  f.scal = f.part + 2 * (size_t)nt * nt;
  f.fallback = reinterpret_cast<int *>(f.scal + 4);
  return f;
}

KS_DEVICE int dsf_active(const DSFArgs &f) { return (f.st ? f.st->m : f.n) - f.l; }

// a signed integer key with the order of the double (NaN-free input): negative values have all bits below the sign
// flipped
KS_DEVICE long long dsf_order_key(double x) {
  const long long b = __double_as_longlong(x);
  return b >= 0 ? b : (b ^ 0x7fffffffffffffffLL);
}

// Dense T of the active block from the compact storage: diagonal d; couplings e[i] for i in [l, n-1), between
// rows i and k when i < k (arrow, raw form) and between rows i and i+1 otherwise.
__global__ void k_dsf_build(DSFArgs f) {
  const int m = dsf_active(f), l = f.l, k = f.k, ld = f.ld;
  if (blockIdx.x == 0 && threadIdx.x == 0) *f.fallback = 0;
  for (int idx = threadIdx.x + blockIdx.x * blockDim.x; idx < m * m; idx += blockDim.x * gridDim.x) {
    const int i = idx % m, j = idx / m;
    const int gi = i + l, gj = j + l;
    double v = 0.0;
    if (gi == gj) v = f.d[gi];
    else {
      const int lo = gi < gj ? gi : gj, hi = gi < gj ? gj : gi;
      if (f.raw && lo < k) { if (hi == k) v = f.e[lo]; }
      else if (hi == lo + 1) v = f.e[lo];
    }
    f.T[i + (size_t)j * ld] = v;
  }
}

// r = hypot(f, g), s = f / r, c = g / r with one reciprocal square root; the slow path covers under/overflow
KS_DEVICE void dsf_rot(float f, float g, float &c, float &s, float &r) {
  const float t = fmaf(f, f, g * g);
  if (t > 1e-30f && t < 1e30f) {
    const float ir = rsqrtf(t);
    r = t * ir;
    s = f * ir;
    c = g * ir;
  } else {
    r = hypotf(f, g);
    if (r != 0.0f) { s = f / r; c = g / r; }
    else { s = 0.0f; c = 1.0f; }
  }
}

KS_DEVICE void dsf_givens(float f, float g, float &c, float &s, float &r) {
  if (g == 0.0f) { c = 1.0f; s = 0.0f; r = f; }
  else if (f == 0.0f) { c = 0.0f; s = copysignf(1.0f, g); r = fabsf(g); }
  else { const float dd = hypotf(f, g); c = fabsf(f) / dd; r = copysignf(dd, f); s = g / r; }
}

// FP32 eigendecomposition of the active block: X0 (m x m, leading dimension ld) and the QL failure flag.
__global__ void __launch_bounds__(DSF_THREADS, 1) k_dsf_eig32(DSFArgs f) {
  extern __shared__ float Xs[];  // m x m, column-major, leading dimension m
  __shared__ float sd[DSF_MAXN], se[DSF_MAXN], rc[DSF_MAXN], rs[DSF_MAXN];
  __shared__ int s_cmd, s_lo, s_hi, s_fail;
  const int tid = threadIdx.x;
  const int m = dsf_active(f), l = f.l, k = f.k;
  for (int i = tid; i < m; i += DSF_THREADS) {
    sd[i] = (float)f.d[l + i];
    se[i] = (float)f.e[l + i];
  }
  for (int i = tid; i < m * m; i += DSF_THREADS) Xs[i] = ((i % m) == (i / m)) ? 1.0f : 0.0f;
  if (tid == 0) s_fail = 0;
  __syncthreads();
  // arrowhead block [0, k-l] -> tridiagonal, rotations chased to the top-left corner (DSArrowTridiag)
  const int n1 = f.raw ? k - l + 1 : 0;
  for (int j = 0; j < n1 - 2; ++j) {
    if (tid == 0) {
      float *d = sd, *e = se;
      float c, s, r;
      dsf_givens(e[j + 1], e[j], c, s, r);
      e[j + 1] = r;
      s = -s;
      const float dj = d[j], dj1 = d[j + 1];
      e[j] = c * s * (dj1 - dj);
      d[j + 1] = s * s * dj + c * c * dj1;
      d[j] = c * c * dj + s * s * dj1;
      rc[0] = c;
      rs[0] = s;
      int t = 1;
      for (int i = j - 1; i >= 0; --i, ++t) {
        const float off = -s * e[i];
        e[i] = c * e[i];
        dsf_givens(e[i + 1], off, c, s, r);
        e[i + 1] = r;
        s = -s;
        const float tt = (d[i] - d[i + 1]) * s - 2.0f * c * e[i];
        const float p = s * tt;
        d[i + 1] += p;
        d[i] -= p;
        e[i] = -e[i] - c * tt;
        rc[t] = c;
        rs[t] = s;
      }
    }
    __syncthreads();
    for (int r = tid; r < j + 2; r += DSF_THREADS) {
      float *row = Xs + r;
      for (int t = 0; t <= j; ++t) {
        const int p = (t == 0) ? j : j - t;
        const float c = rc[t], s = rs[t];
        float *x = row + (size_t)p * m, *y = row + (size_t)(p + 1) * m;
        const float xv = *x, yv = *y;
        *x = c * xv + s * yv;
        *y = c * yv - s * xv;
      }
    }
    __syncthreads();
  }
  // implicit QL with Wilkinson shifts: thread 0 computes a sweep, every thread applies it to its row of X
  {
    int ll = 0, total = 0;
    float *d = sd, *e = se;
    if (tid == 0 && m > 0) e[m - 1] = 0.0f;
    for (;;) {
      if (tid == 0) {
        s_cmd = 0;
        while (ll < m) {
          int mm;
          for (mm = ll; mm < m - 1; ++mm) {
            const float dd = fabsf(d[mm]) + fabsf(d[mm + 1]);
            if (fabsf(e[mm]) <= FLT_EPSILON * dd) break;
          }
          if (mm == ll) { ++ll; continue; }
          if (++total > 30 * m) { s_fail = 1; break; }
          float g = (d[ll + 1] - d[ll]) / (2.0f * e[ll]);
          float r = hypotf(g, 1.0f);
          g = d[mm] - d[ll] + e[ll] / (g + copysignf(r, g));
          float s = 1.0f, c = 1.0f, p = 0.0f;
          int i, under = 0;
          for (i = mm - 1; i >= ll; --i) {
            const float ff = s * e[i], b = c * e[i];
            dsf_rot(ff, g, c, s, r);
            e[i + 1] = r;
            if (r == 0.0f) { d[i + 1] -= p; e[mm] = 0.0f; under = 1; break; }
            g = d[i + 1] - p;
            r = (d[i] - g) * s + 2.0f * c * b;
            p = s * r;
            d[i + 1] = g + p;
            g = c * r - b;
            rc[i] = c;
            rs[i] = s;
          }
          if (!under) { d[ll] -= p; e[ll] = g; e[mm] = 0.0f; }
          s_lo = under ? i + 1 : ll;
          s_hi = mm;
          s_cmd = 1;
          break;
        }
      }
      __syncthreads();
      if (s_cmd == 0) break;
      const int lo = s_lo, hi = s_hi;
      for (int r = tid; r < m; r += DSF_THREADS) {
        float *row = Xs + r;
        float carry = row[(size_t)hi * m];
        for (int i = hi - 1; i >= lo; --i) {
          const float c = rc[i], s = rs[i];
          const float x = row[(size_t)i * m];
          row[(size_t)(i + 1) * m] = s * x + c * carry;
          carry = c * x - s * carry;
        }
        row[(size_t)lo * m] = carry;
      }
      __syncthreads();
    }
  }
  for (int i = tid; i < m * m; i += DSF_THREADS) f.X[(i % m) + (size_t)(i / m) * f.ld] = (double)Xs[i];
  if (tid == 0 && f.ctl) f.ctl->ds_error = s_fail;
}

// ---- small FP64 products: 16 x 16 output tile per block, thread (ty, tx) owns output (i0 + ty, j0 + tx) ----

enum { DSF_MM_TX = 0, DSF_MM_SG = 1, DSF_MM_UPDATE = 2, DSF_MM_NS = 3 };

// DSF_MM_TX:     C = A B                        (P = T X)
// DSF_MM_SG:     C = A^T B, C2 = A^T A          (S = X^T P, G = X^T X), plus the block partial sums of
//                ||S - diag(s_ii / g_ii)||_F^2 and ||I - G||_F^2 in f.part
// DSF_MM_UPDATE: C = A + A E, E formed on the fly from S, G, lambda and the threshold in f.scal[0]
// DSF_MM_NS:     C = 1.5 A - 0.5 A B            (Newton-Schulz with B = X^T X)
template <int MODE>
__global__ void __launch_bounds__(256) k_dsf_mm(DSFArgs f, const double *A, const double *B, double *C, double *C2) {
  __shared__ double As[DSF_TILE][DSF_TILE + 1], Bs[DSF_TILE][DSF_TILE + 1], Bs2[DSF_TILE][DSF_TILE + 1];
  __shared__ double red[8][2];
  const int m = dsf_active(f), ld = f.ld;
  const int tx = threadIdx.x % DSF_TILE, ty = threadIdx.x / DSF_TILE;
  const int i0 = blockIdx.y * DSF_TILE, j0 = blockIdx.x * DSF_TILE;
  if (i0 >= m || j0 >= m) return;  // whole blocks only
  const int i = i0 + ty, j = j0 + tx;
  double thr = 0.0;
  if (MODE == DSF_MM_UPDATE) thr = f.scal[0];
  double acc = 0.0, acc2 = 0.0;
  for (int k0 = 0; k0 < m; k0 += DSF_TILE) {
    // A operand tile As[r][c] = op(A)(i0 + r, k0 + c)
    double av = 0.0;
    if (i < m && k0 + tx < m) {
      if (MODE == DSF_MM_SG) av = A[(k0 + tx) + (size_t)i * ld];
      else av = A[i + (size_t)(k0 + tx) * ld];
    }
    As[ty][tx] = av;
    // B operand tile Bs[r][c] = B(k0 + r, j0 + c)
    const int kr = k0 + ty;
    double bv = 0.0, bv2 = 0.0;
    if (kr < m && j < m) {
      const size_t o = kr + (size_t)j * ld;
      if (MODE == DSF_MM_UPDATE) {
        const double lj = f.lam[j], lk = f.lam[kr];
        const double rr = (kr == j ? 1.0 : 0.0) - f.G[o];
        const double gap = lj - lk;
        bv = (fabs(gap) > thr) ? (f.S[o] + lj * rr) / gap : 0.5 * rr;
      } else {
        bv = B[o];
        if (MODE == DSF_MM_SG) bv2 = A[o];
      }
    }
    Bs[ty][tx] = bv;
    if (MODE == DSF_MM_SG) Bs2[ty][tx] = bv2;
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < DSF_TILE; ++kk) {
      acc = fma(As[ty][kk], Bs[kk][tx], acc);
      if (MODE == DSF_MM_SG) acc2 = fma(As[ty][kk], Bs2[kk][tx], acc2);
    }
    __syncthreads();
  }
  const bool in = i < m && j < m;
  const size_t o = i + (size_t)j * ld;
  if (MODE == DSF_MM_TX) {
    if (in) C[o] = acc;
  } else if (MODE == DSF_MM_UPDATE) {
    if (in) C[o] = A[o] + acc;
  } else if (MODE == DSF_MM_NS) {
    if (in) C[o] = 1.5 * A[o] - 0.5 * acc;
  } else {
    double p0 = 0.0, p1 = 0.0;
    if (in) {
      C[o] = acc;
      C2[o] = acc2;
      const double sv = (i == j) ? acc - acc / acc2 : acc;
      const double rv = (i == j ? 1.0 : 0.0) - acc2;
      p0 = sv * sv;
      p1 = rv * rv;
    }
    for (int off = 16; off > 0; off >>= 1) {
      p0 += __shfl_down_sync(0xffffffffu, p0, off);
      p1 += __shfl_down_sync(0xffffffffu, p1, off);
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) { red[warp][0] = p0; red[warp][1] = p1; }
    __syncthreads();
    if (threadIdx.x == 0) {
      double q0 = 0.0, q1 = 0.0;
      for (int w = 0; w < 8; ++w) { q0 += red[w][0]; q1 += red[w][1]; }
      const int b = blockIdx.y * gridDim.x + blockIdx.x;
      f.part[2 * b] = q0;
      f.part[2 * b + 1] = q1;
    }
  }
}

// cyclic Jacobi on one cluster block of S (one thread); A and W are len x len with leading dimension lda
KS_DEVICE void dsf_jacobi(int len, double *A, double *W, int lda) {
  for (int q = 0; q < len; ++q)
    for (int p = 0; p < len; ++p) W[p + (size_t)q * lda] = (p == q) ? 1.0 : 0.0;
  for (int sweep = 0; sweep < 30; ++sweep) {
    double off = 0.0, nrm = 0.0;
    for (int q = 0; q < len; ++q)
      for (int p = 0; p < len; ++p) {
        const double v = A[p + (size_t)q * lda];
        nrm += v * v;
        if (p != q) off += v * v;
      }
    if (off == 0.0 || off <= 1e-32 * nrm) break;
    for (int p = 0; p < len - 1; ++p)
      for (int q = p + 1; q < len; ++q) {
        const double apq = A[p + (size_t)q * lda];
        if (apq == 0.0) continue;
        const double tau = (A[q + (size_t)q * lda] - A[p + (size_t)p * lda]) / (2.0 * apq);
        const double t = (tau >= 0.0 ? 1.0 : -1.0) / (fabs(tau) + sqrt(1.0 + tau * tau));
        const double c = 1.0 / sqrt(1.0 + t * t), sn = t * c;
        for (int r = 0; r < len; ++r) {  // columns p, q
          const double ap = A[r + (size_t)p * lda], aq = A[r + (size_t)q * lda];
          A[r + (size_t)p * lda] = c * ap - sn * aq;
          A[r + (size_t)q * lda] = sn * ap + c * aq;
        }
        for (int r = 0; r < len; ++r) {  // rows p, q
          const double ap = A[p + (size_t)r * lda], aq = A[q + (size_t)r * lda];
          A[p + (size_t)r * lda] = c * ap - sn * aq;
          A[q + (size_t)r * lda] = sn * ap + c * aq;
        }
        for (int r = 0; r < len; ++r) {
          const double wp = W[r + (size_t)p * lda], wq = W[r + (size_t)q * lda];
          W[r + (size_t)p * lda] = c * wp - sn * wq;
          W[r + (size_t)q * lda] = sn * wp + c * wq;
        }
      }
  }
}

// The scalar part of one refinement step (one block): lambda, delta, the threshold, clusters and their rotations.
__global__ void __launch_bounds__(DSF_THREADS, 1) k_dsf_step(DSFArgs f, int final_pass) {
  __shared__ double lam[DSF_MAXN], red[DSF_THREADS / 32][4];
  __shared__ int by_rank[DSF_MAXN], close_next[DSF_MAXN], cl_start[DSF_MAXN], cl_len[DSF_MAXN], cl_of[DSF_MAXN];
  __shared__ int s_ncl;
  __shared__ double s_tau, s_tnorm;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int m = dsf_active(f), ld = f.ld, l = f.l;
  double *S = f.S, *G = f.G, *X = f.X;
  const int nt = (m + DSF_TILE - 1) / DSF_TILE;
  // lambda, ||T||_F^2, the block partial sums of the product kernel, max |lambda|
  double a0 = 0.0, a1 = 0.0, a2 = 0.0, amax = 0.0;
  for (int i = tid; i < m; i += DSF_THREADS) {
    const double li = S[i + (size_t)i * ld] / G[i + (size_t)i * ld];
    lam[i] = li;
    amax = fmax(amax, fabs(li));
    const double di = f.d[l + i];
    a2 += di * di;
    if (i < m - 1) a2 += 2.0 * f.e[l + i] * f.e[l + i];
  }
  for (int b = tid; b < nt * nt; b += DSF_THREADS) {
    a0 += f.part[2 * b];
    a1 += f.part[2 * b + 1];
  }
  for (int off = 16; off > 0; off >>= 1) {
    a0 += __shfl_down_sync(0xffffffffu, a0, off);
    a1 += __shfl_down_sync(0xffffffffu, a1, off);
    a2 += __shfl_down_sync(0xffffffffu, a2, off);
    amax = fmax(amax, __shfl_down_sync(0xffffffffu, amax, off));
  }
  if (lane == 0) { red[warp][0] = a0; red[warp][1] = a1; red[warp][2] = a2; red[warp][3] = amax; }
  __syncthreads();
  // ascending ranks (ties by index)
  for (int i = tid; i < m; i += DSF_THREADS) {
    int r = 0;
    const double li = lam[i];
    for (int j = 0; j < m; ++j) r += (lam[j] < li) || (lam[j] == li && j < i);
    by_rank[r] = i;
  }
  if (tid == 0) {
    double b0 = 0.0, b1 = 0.0, b2 = 0.0, bm = 0.0;
    for (int w = 0; w < DSF_THREADS / 32; ++w) {
      b0 += red[w][0]; b1 += red[w][1]; b2 += red[w][2]; bm = fmax(bm, red[w][3]);
    }
    const double tau = DSF_TAU * bm;
    s_tnorm = sqrt(b2);
    const double delta = 2.0 * (sqrt(b0) + sqrt(b2) * sqrt(b1));
    // pairs closer than max(delta, tau) get no first-order correction in the update: they are clustered, so the
    // cluster pass diagonalises them (the clustered-eigenvalue form of the refinement); a fixed tau alone left pairs
    // between tau and delta neither corrected nor rotated
    s_tau = fmax(delta, tau);
    if (!final_pass) f.scal[0] = fmax(delta, tau);
  }
  __syncthreads();
  const double tau = s_tau;
  for (int r = tid; r < m; r += DSF_THREADS)
    close_next[r] = (r + 1 < m) && (lam[by_rank[r + 1]] - lam[by_rank[r]] <= tau);
  __syncthreads();
  if (tid == 0) {
    int ncl = 0, i = 0;
    while (i < m) {
      int j = i;
      while (close_next[j] && j + 1 - i < DSF_CL) ++j;
      if (j > i) { cl_start[ncl] = i; cl_len[ncl] = j - i + 1; ++ncl; }
      i = j + 1;
    }
    s_ncl = ncl;
  }
  __syncthreads();
  const int ncl = s_ncl;
  if (final_pass) {
    // Accuracy check of the refined pairs: outside the clusters (diagonalised next by FP64 Jacobi) every
    // off-diagonal entry of S = X^T T X must be at rounding level of ||T||, and G = X^T X close enough to I for the
    // Newton-Schulz step.
    // A pair whose gap is too small for the refinement to converge in DSF_ITERS steps stays mixed and fails here;
    // the FP64 QR solver (k_ds_hep) then redoes the whole projected problem.
    for (int i = tid; i < m; i += DSF_THREADS) cl_of[i] = -1;
    __syncthreads();
    for (int c = 0; c < ncl; ++c)
      for (int q = tid; q < cl_len[c]; q += DSF_THREADS) cl_of[by_rank[cl_start[c] + q]] = c;
    __syncthreads();
    double ms = 0.0, mg = 0.0;
    for (int idx = tid; idx < m * m; idx += DSF_THREADS) {
      const int i = idx % m, j = idx / m;
      const double g = G[i + (size_t)j * ld] - (i == j ? 1.0 : 0.0);
      mg = fmax(mg, fabs(g));
      if (i != j && !(cl_of[i] >= 0 && cl_of[i] == cl_of[j])) ms = fmax(ms, fabs(S[i + (size_t)j * ld]));
    }
    for (int off = 16; off > 0; off >>= 1) {
      ms = fmax(ms, __shfl_down_sync(0xffffffffu, ms, off));
      mg = fmax(mg, __shfl_down_sync(0xffffffffu, mg, off));
    }
    if (lane == 0) { red[warp][0] = ms; red[warp][1] = mg; }
    __syncthreads();
    if (tid == 0) {
      double bs = 0.0, bg = 0.0;
      for (int w = 0; w < DSF_THREADS / 32; ++w) { bs = fmax(bs, red[w][0]); bg = fmax(bg, red[w][1]); }
      const int bad = !(bs <= DSF_CHECK * DBL_EPSILON * s_tnorm) || !(bg <= DSF_CHECK_G);
      *f.fallback = bad;
      f.ctl->ds_fallback = bad;
    }
    __syncthreads();
  }
  if (ncl > 0) {
    // one thread per cluster: Jacobi on the symmetrised block of S; W and the block copy live in f.W, indexed
    // by rank (rows s0 .. s0+len-1 of an ld x DSF_CL array), so clusters never overlap
    double *Wb = f.W, *Ab = f.W + (size_t)ld * DSF_CL;
    for (int c = tid; c < ncl; c += DSF_THREADS) {
      const int s0 = cl_start[c], len = cl_len[c];
      for (int q = 0; q < len; ++q)
        for (int p = 0; p < len; ++p) {
          const int gp = by_rank[s0 + p], gq = by_rank[s0 + q];
          Ab[(s0 + p) + (size_t)q * ld] = 0.5 * (S[gp + (size_t)gq * ld] + S[gq + (size_t)gp * ld]);
        }
      dsf_jacobi(len, Ab + s0, Wb + s0, ld);
    }
    __syncthreads();
    // columns of X, S, G in each cluster times W (rows in parallel)
    for (int r = tid; r < m; r += DSF_THREADS) {
      for (int c = 0; c < ncl; ++c) {
        const int s0 = cl_start[c], len = cl_len[c];
        double tx[DSF_CL], ts[DSF_CL], tg[DSF_CL];
        for (int q = 0; q < len; ++q) {
          double ax = 0.0, as = 0.0, ag = 0.0;
          for (int p = 0; p < len; ++p) {
            const size_t gp = (size_t)by_rank[s0 + p] * ld + r;
            const double w = Wb[(s0 + p) + (size_t)q * ld];
            ax = fma(X[gp], w, ax);
            as = fma(S[gp], w, as);
            ag = fma(G[gp], w, ag);
          }
          tx[q] = ax; ts[q] = as; tg[q] = ag;
        }
        for (int q = 0; q < len; ++q) {
          const size_t gq = (size_t)by_rank[s0 + q] * ld + r;
          X[gq] = tx[q]; S[gq] = ts[q]; G[gq] = tg[q];
        }
      }
    }
    __syncthreads();
    // rows of S, G in each cluster: W^T times them (columns in parallel)
    for (int cc = tid; cc < m; cc += DSF_THREADS) {
      for (int c = 0; c < ncl; ++c) {
        const int s0 = cl_start[c], len = cl_len[c];
        double ts[DSF_CL], tg[DSF_CL];
        for (int q = 0; q < len; ++q) {
          double as = 0.0, ag = 0.0;
          for (int p = 0; p < len; ++p) {
            const size_t gp = by_rank[s0 + p] + (size_t)cc * ld;
            const double w = Wb[(s0 + p) + (size_t)q * ld];
            as = fma(w, S[gp], as);
            ag = fma(w, G[gp], ag);
          }
          ts[q] = as; tg[q] = ag;
        }
        for (int q = 0; q < len; ++q) {
          const size_t gq = by_rank[s0 + q] + (size_t)cc * ld;
          S[gq] = ts[q]; G[gq] = tg[q];
        }
      }
    }
    __syncthreads();
    for (int c = 0; c < ncl; ++c)
      for (int q = tid; q < cl_len[c]; q += DSF_THREADS) {
        const int g = by_rank[cl_start[c] + q];
        lam[g] = S[g + (size_t)g * ld] / G[g + (size_t)g * ld];
      }
    __syncthreads();
  }
  for (int i = tid; i < m; i += DSF_THREADS) f.lam[i] = lam[i];
}

// Sort by the criterion, write Q (identity on the locked block), d, the extra row, the error estimates and the
// restart control record (the tail of EPSSolve_KrylovSchur_Default for the symmetric case, krylovschur.c:270-322).
__global__ void __launch_bounds__(DSF_THREADS, 1) k_dsf_finish(DSFArgs f, DSArgs a) {
  if (*f.fallback) return;  // the FP64 QR solver redoes this projected problem (launched next)
  __shared__ double lam[DSF_MAXN], serr[DSF_MAXN];
  __shared__ long long k_crit[DSF_MAXN], k_asc[DSF_MAXN];
  __shared__ int perm[DSF_MAXN];
  __shared__ double s_beta_e;
  const int tid = threadIdx.x;
  const int m = dsf_active(f), l = f.l, n = m + l, ld = f.ld;
  if (tid == 0) s_beta_e = a.e[n - 1];
  for (int i = tid; i < m; i += DSF_THREADS) lam[i] = f.lam[i];
  __syncthreads();
  // The order of steqr's ascending sort followed by the stable insertion sort by the criterion (dspriv.c:226-245):
  // by the criterion first, ties by ascending value, then by index.  Each thread ranks its own eigenvalue with
  // order-preserving integer keys (k_crit: the criterion's "goes first" order, k_asc: ascending value).
  for (int i = tid; i < m; i += DSF_THREADS) {
    const double v = lam[i] + 0.0;  // -0 -> +0, as the floating-point comparisons treat them
    const double c = (a.which == 1 || a.which == 2) ? fabs(v) : (a.which >= 7 ? fabs(v - a.target) : v);
    const long long kv = dsf_order_key(v), kc0 = dsf_order_key(c);
    k_asc[i] = kv;
    k_crit[i] = (a.which == 1 || a.which == 3) ? ~kc0 : kc0;  // largest first: reversed; targets: nearest first
  }
  __syncthreads();
  for (int i = tid; i < m; i += DSF_THREADS) {
    const long long ci = k_crit[i], ai = k_asc[i];
    int r = 0;
    for (int j = 0; j < m; ++j) {
      const long long cj = k_crit[j], aj = k_asc[j];
      r += (cj < ci) || (cj == ci && (aj < ai || (aj == ai && j < i)));
    }
    perm[r] = i;
  }
  __syncthreads();
  for (int idx = tid; idx < n * n; idx += DSF_THREADS) {
    const int i = idx % n, j = idx / n;
    double v;
    if (i < l || j < l) v = (i == j) ? 1.0 : 0.0;
    else v = f.X[(i - l) + (size_t)perm[j - l] * ld];
    a.Q[i + (size_t)j * a.ld] = v;
  }
  const double beta = a.st ? a.st->beta_out : 0.0;
  const double beta_e = s_beta_e;
  for (int i = tid; i < n; i += DSF_THREADS) {
    const double di = (i < l) ? a.d[i] : lam[perm[i - l]];
    const double qlast = (i < l) ? ((i == n - 1) ? 1.0 : 0.0) : f.X[(m - 1) + (size_t)perm[i - l] * ld];
    const double w = fabs(di);
    serr[i] = ds_conv_errest(a, fabs(qlast) * beta, w);
    a.eigr[i] = di;
    if (a.eigi) a.eigi[i] = 0.0;
  }
  __syncthreads();
  for (int i = tid; i < n; i += DSF_THREADS) {
    const double qlast = (i < l) ? ((i == n - 1) ? 1.0 : 0.0) : f.X[(m - 1) + (size_t)perm[i - l] * ld];
    a.e[i] = beta_e * qlast;
    if (i >= l) a.d[i] = lam[perm[i - l]];
  }
  if (tid == 0) {
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
    const int breakdown = a.st->breakdown;
    int lkeep;
    if (reason != 0 || breakdown || kk == n) lkeep = 0;
    else {
      lkeep = (int)((n - kk) * a.keep);
      if (lkeep < 1) lkeep = 1;
    }
    if (!a.lock && lkeep > 0) { lkeep += kk; kk = 0; }
    const int fail = ctl->ds_error;
    ctl->nconv = kk;
    ctl->l = lkeep;
    ctl->reason = reason;
    ctl->nv = n;
    ctl->breakdown = breakdown;
    ctl->need_start = (reason == 0 && (breakdown || kk == n) && kk < a.nev) ? 1 : 0;
    ctl->ds_error = fail;
    ctl->beta = beta;
  }
}

int ds_fast_launches() { return 2 + 3 * (DSF_ITERS + 1) + DSF_ITERS + 4; }

cudaError_t launch_ds_hep_fast(const DSArgs &a, const DSFArgs &f0, int n_max, cudaStream_t s) {
  if (n_max > DSF_MAXN || f0.ld < n_max || a.ld != f0.ld || !a.st || !a.ctl) return cudaErrorInvalidValue;
  DSFArgs f = f0;
  f.n = a.n;
  f.l = a.l;
  f.k = a.k;
  f.raw = a.raw;
  f.d = a.d;
  f.e = a.e;
  f.st = a.st;
  f.ctl = a.ctl;
  const int mmax = n_max - a.l;
  if (mmax <= 0) return cudaErrorInvalidValue;
  const size_t shm = (size_t)mmax * mmax * sizeof(float);
  cudaError_t err = cudaFuncSetAttribute(k_dsf_eig32, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm);
  if (err != cudaSuccess) return err;
  const int nt = (mmax + DSF_TILE - 1) / DSF_TILE;
  const dim3 grid(nt, nt);
  k_dsf_build<<<16, 256, 0, s>>>(f);
  k_dsf_eig32<<<1, DSF_THREADS, shm, s>>>(f);
  for (int it = 0; it <= DSF_ITERS; ++it) {
    const int final_pass = (it == DSF_ITERS);
    k_dsf_mm<DSF_MM_TX><<<grid, 256, 0, s>>>(f, f.T, f.X, f.P, nullptr);
    k_dsf_mm<DSF_MM_SG><<<grid, 256, 0, s>>>(f, f.X, f.P, f.S, f.G);
    k_dsf_step<<<1, DSF_THREADS, 0, s>>>(f, final_pass);
    if (!final_pass) {
      k_dsf_mm<DSF_MM_UPDATE><<<grid, 256, 0, s>>>(f, f.X, nullptr, f.P, nullptr);
      double *t = f.X; f.X = f.P; f.P = t;
    }
  }
  // Newton-Schulz: G = X^T X (S = X^T X as well, unused), X <- 1.5 X - 0.5 X G
  k_dsf_mm<DSF_MM_SG><<<grid, 256, 0, s>>>(f, f.X, f.X, f.S, f.G);
  k_dsf_mm<DSF_MM_NS><<<grid, 256, 0, s>>>(f, f.X, f.G, f.P, nullptr);
  { double *t = f.X; f.X = f.P; f.P = t; }
  k_dsf_finish<<<1, DSF_THREADS, 0, s>>>(f, a);
  // the fallback: the reference's FP64 algorithm on the untouched compact form, only when the check failed
  DSArgs q = a;
  q.run_if = f.fallback;
  return launch_ds_hep(q, n_max, s);
}

}  // namespace ksg
