// k_dense.cu -- the operator of a generalised problem with a non-diagonal B: C = B^-1 A, formed once at set-up.
//
// EPSSetUp with B (STSHIFT with B and a direct solve, epssetup.c:321-353 and the ST's KSP of type preonly + LU) asks
// for B^-1 A at every Krylov step.  For the problem sizes that path serves (n <= 2048, B dense on the device) the
// product is formed once: B is factorised P B = L U with partial pivoting (the algorithm of LAPACK's getrf, right-
// looking, one thread block), then the n right-hand sides of B C = A are solved one per thread (getrs: the row
// interchanges, the unit lower and the upper triangular solve), all in FP64.  The Krylov iteration then runs on C
// as on any operator.  Row-major storage throughout: a row swap is contiguous, and for a fixed row the threads of a
// solve read consecutive columns.
#include "common.cuh"
#include "kernels.h"

namespace ksg {

constexpr int DN_THREADS = 1024;

// dense row-major copy of a CSR matrix (one block per row; duplicate entries add up, as in MatSetValues ADD)
__global__ void k_csr_to_dense_rm(const int *__restrict__ rp, const int *__restrict__ ci,
                                  const double *__restrict__ va, int n, double *__restrict__ D) {
  for (int r = blockIdx.x; r < n; r += gridDim.x) {
    double *row = D + (size_t)r * n;
    for (int c = threadIdx.x; c < n; c += blockDim.x) row[c] = 0.0;
    __syncthreads();
    if (threadIdx.x == 0)
      for (int p = rp[r]; p < rp[r + 1]; ++p) row[ci[p]] += va[p];
    __syncthreads();
  }
}

// P B = L U in place (row-major, unit L below the diagonal), piv[k] = the row swapped with row k; *err = k + 1 at
// the first exactly zero pivot (B singular)
__global__ void __launch_bounds__(DN_THREADS) k_lu_rm(double *__restrict__ B, int n, int *__restrict__ piv,
                                                      int *__restrict__ err) {
  __shared__ double sv[DN_THREADS / 32];
  __shared__ int si[DN_THREADS / 32];
  __shared__ int s_p;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int k = 0; k < n; ++k) {
    // pivot: the largest |B(i, k)|, i >= k (the first one among equals, as idamax)
    double bv = -1.0;
    int bi = n;
    for (int i = k + tid; i < n; i += DN_THREADS) {
      const double v = fabs(B[(size_t)i * n + k]);
      if (v > bv) { bv = v; bi = i; }
    }
    for (int o = 16; o > 0; o >>= 1) {
      const double ov = __shfl_down_sync(0xffffffffu, bv, o);
      const int oi = __shfl_down_sync(0xffffffffu, bi, o);
      if (ov > bv || (ov == bv && oi < bi)) { bv = ov; bi = oi; }
    }
    if (lane == 0) { sv[warp] = bv; si[warp] = bi; }
    __syncthreads();
    if (tid == 0) {
      double v = sv[0];
      int p = si[0];
      for (int w = 1; w < DN_THREADS / 32; ++w)
        if (sv[w] > v || (sv[w] == v && si[w] < p)) { v = sv[w]; p = si[w]; }
      s_p = (v > 0.0) ? p : -1;
      piv[k] = p < n ? p : k;
      if (s_p < 0 && *err == 0) *err = k + 1;
    }
    __syncthreads();
    const int p = s_p;
    if (p < 0) return;  // singular: the caller reports it
    if (p != k)
      for (int c = tid; c < n; c += DN_THREADS) {
        const double t = B[(size_t)k * n + c];
        B[(size_t)k * n + c] = B[(size_t)p * n + c];
        B[(size_t)p * n + c] = t;
      }
    __syncthreads();
    const double inv = 1.0 / B[(size_t)k * n + k];
    for (int i = k + 1 + tid; i < n; i += DN_THREADS) B[(size_t)i * n + k] *= inv;
    __syncthreads();
    const int m = n - k - 1;
    for (long long t = tid; t < (long long)m * m; t += DN_THREADS) {
      const int i = k + 1 + (int)(t / m), c = k + 1 + (int)(t % m);
      B[(size_t)i * n + c] = fma(-B[(size_t)i * n + k], B[(size_t)k * n + c], B[(size_t)i * n + c]);
    }
    __syncthreads();
  }
}

// X <- B^-1 X for the factors of k_lu_rm: thread c solves column c of the row-major n x m X (nothing after a zero
// pivot: the factors and interchanges are incomplete then)
__global__ void k_lu_solve_cols(const double *__restrict__ LU, const int *__restrict__ piv, double *__restrict__ X,
                                int n, int m, const int *__restrict__ err) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m || *err) return;
  for (int k = 0; k < n; ++k) {
    const int p = piv[k];
    if (p != k) {
      const double t = X[(size_t)k * m + c];
      X[(size_t)k * m + c] = X[(size_t)p * m + c];
      X[(size_t)p * m + c] = t;
    }
  }
  for (int i = 1; i < n; ++i) {  // L y = P x, unit diagonal
    double s = X[(size_t)i * m + c];
    const double *l = LU + (size_t)i * n;
    for (int j = 0; j < i; ++j) s = fma(-l[j], X[(size_t)j * m + c], s);
    X[(size_t)i * m + c] = s;
  }
  for (int i = n - 1; i >= 0; --i) {  // U x = y
    double s = X[(size_t)i * m + c];
    const double *u = LU + (size_t)i * n;
    for (int j = i + 1; j < n; ++j) s = fma(-u[j], X[(size_t)j * m + c], s);
    X[(size_t)i * m + c] = s / u[i];
  }
}

// B = L L^T in place (row-major, L in the lower triangle); *err = k + 1 when the k-th pivot is not positive (B not
// positive definite)
__global__ void __launch_bounds__(DN_THREADS) k_chol_rm(double *__restrict__ B, int n, int *__restrict__ err) {
  __shared__ double s_d;
  const int tid = threadIdx.x;
  for (int k = 0; k < n; ++k) {
    if (tid == 0) {
      const double p = B[(size_t)k * n + k];
      s_d = (p > 0.0) ? sqrt(p) : -1.0;
      if (s_d < 0.0 && *err == 0) *err = k + 1;
    }
    __syncthreads();
    const double dk = s_d;
    if (dk < 0.0) return;
    if (tid == 0) B[(size_t)k * n + k] = dk;
    const double inv = 1.0 / dk;
    for (int i = k + 1 + tid; i < n; i += DN_THREADS) B[(size_t)i * n + k] *= inv;
    __syncthreads();
    // the trailing lower triangle: B(i, c) -= L(i, k) L(c, k), k < c <= i
    const int m = n - k - 1;
    for (long long t = tid; t < (long long)m * m; t += DN_THREADS) {
      const int i = k + 1 + (int)(t / m), c = k + 1 + (int)(t % m);
      if (c <= i) B[(size_t)i * n + c] = fma(-B[(size_t)i * n + k], B[(size_t)c * n + k], B[(size_t)i * n + c]);
    }
    __syncthreads();
  }
}

// X <- L^-1 X (L lower, row-major): thread c solves column c of the row-major n x m X
__global__ void k_lower_solve_cols(const double *__restrict__ L, double *__restrict__ X, int n, int m,
                                   const int *__restrict__ err) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m || *err) return;
  for (int i = 0; i < n; ++i) {
    double s = X[(size_t)i * m + c];
    const double *l = L + (size_t)i * n;
    for (int j = 0; j < i; ++j) s = fma(-l[j], X[(size_t)j * m + c], s);
    X[(size_t)i * m + c] = s / l[i];
  }
}

__global__ void k_transpose_sq(const double *__restrict__ X, double *__restrict__ Y, int n) {
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < (long long)n * n;
       t += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(t / n), j = (int)(t % n);
    Y[(size_t)j * n + i] = X[t];
  }
}

// C <- (C + C^T) / 2: the operator of a symmetric pencil exactly symmetric
__global__ void k_symmetrize_sq(double *__restrict__ C, int n) {
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < (long long)n * n;
       t += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(t / n), j = (int)(t % n);
    if (j > i) {
      const double v = 0.5 * (C[t] + C[(size_t)j * n + i]);
      C[t] = v;
      C[(size_t)j * n + i] = v;
    }
  }
}

// y = L^T x (L lower, row-major): thread i sums L(j, i) x_j over j >= i
__global__ void k_lt_mv(const double *__restrict__ L, const double *__restrict__ x, double *__restrict__ y, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int j = i; j < n; ++j) s = fma(L[(size_t)j * n + i], x[j], s);
    y[i] = s;
  }
}

// X <- L^-T X for m column-major right-hand sides (leading dimension ldx): thread c back-substitutes column c
__global__ void k_lt_solve_cols_cm(const double *__restrict__ L, double *__restrict__ X, int n, int m, long long ldx) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m) return;
  double *x = X + (size_t)c * ldx;
  for (int i = n - 1; i >= 0; --i) {
    double s = x[i];
    for (int j = i + 1; j < n; ++j) s = fma(-L[(size_t)j * n + i], x[j], s);
    x[i] = s / L[(size_t)i * n + i];
  }
}

cudaError_t launch_general_b_ghep(const int *arp, const int *aci, const double *ava, const int *brp, const int *bci,
                                  const double *bva, int n, double *Ld, double *Cd, double *Td, int *err,
                                  cudaStream_t s) {
  if (n <= 0 || n > general_b_max_n()) return cudaErrorInvalidValue;
  const int g = n < 1024 ? n : 1024;
  const int gs = (int)(((long long)n * n + 255) / 256 < 4096 ? ((long long)n * n + 255) / 256 : 4096);
  k_csr_to_dense_rm<<<g, 256, 0, s>>>(brp, bci, bva, n, Ld);
  k_csr_to_dense_rm<<<g, 256, 0, s>>>(arp, aci, ava, n, Cd);
  k_chol_rm<<<1, DN_THREADS, 0, s>>>(Ld, n, err);
  k_lower_solve_cols<<<(n + 127) / 128, 128, 0, s>>>(Ld, Cd, n, n, err);  // L^-1 A
  k_transpose_sq<<<gs, 256, 0, s>>>(Cd, Td, n);                           // (L^-1 A)^T = A L^-T
  k_lower_solve_cols<<<(n + 127) / 128, 128, 0, s>>>(Ld, Td, n, n, err);  // L^-1 A L^-T (A symmetric)
  k_symmetrize_sq<<<gs, 256, 0, s>>>(Td, n);
  return cudaGetLastError();
}

cudaError_t launch_lt_mv(const double *L, const double *x, double *y, int n, cudaStream_t s) {
  k_lt_mv<<<(n + 127) / 128, 128, 0, s>>>(L, x, y, n);
  return cudaGetLastError();
}

cudaError_t launch_lt_solve(const double *L, double *X, int n, int m, long long ldx, cudaStream_t s) {
  if (m <= 0) return cudaSuccess;
  k_lt_solve_cols_cm<<<(m + 127) / 128, 128, 0, s>>>(L, X, n, m, ldx);
  return cudaGetLastError();
}

cudaError_t launch_general_b_operator(const int *arp, const int *aci, const double *ava, const int *brp,
                                      const int *bci, const double *bva, int n, double *Bd, double *Cd, int *piv,
                                      int *err, cudaStream_t s) {
  if (n <= 0 || n > general_b_max_n()) return cudaErrorInvalidValue;
  const int g = n < 1024 ? n : 1024;
  k_csr_to_dense_rm<<<g, 256, 0, s>>>(brp, bci, bva, n, Bd);
  k_csr_to_dense_rm<<<g, 256, 0, s>>>(arp, aci, ava, n, Cd);
  k_lu_rm<<<1, DN_THREADS, 0, s>>>(Bd, n, piv, err);
  k_lu_solve_cols<<<(n + 127) / 128, 128, 0, s>>>(Bd, piv, Cd, n, n, err);
  return cudaGetLastError();
}

int general_b_max_n() { return 2048; }

}  // namespace ksg
