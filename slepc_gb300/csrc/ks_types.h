// ks_types.h -- structures shared by the host driver and the CUDA kernels of the Krylov-Schur path.
#pragma once

#include <stdint.h>

namespace ksg {

struct GTArgs;

// Arithmetic used by the bandwidth-bound kernels (Gram-Schmidt, restart, residual norms).
enum Arith : int {
  ARITH_PAIR = 0,  // FP64 storage, products and sums on FP32 pairs with error-free transformations
  ARITH_F64 = 1,   // FP64 storage, IEEE FP64 FMA (exact reference arithmetic, FP64-pipe bound on GB300)
  ARITH_F32 = 2,   // the precision form: FP32 values and basis with pair accumulation, then an FP64-class sweep
};

// Storage format of the Krylov basis.
enum Storage : int {
  STORE_F64 = 0,   // IEEE doubles
  STORE_PAIR = 1,  // FP32 pairs (hi, lo), value hi + lo: 47-bit significand in 8 bytes
  STORE_F32 = 2,   // FP32 (the precision form's first phase: half the bytes, exact widening into pairs)
};

// Per-factorisation state of the delayed-reorthogonalisation Gram-Schmidt (device resident).
// The raw vector stored in V[:, j] at the start of step j is u_raw; the unit vector it stands for is
// u = sigma * u_raw, already orthogonalised once against V[:, 0:j].
struct KrylovState {
  double sigma;      // scale of u_raw
  double beta_prev;  // ||w'|| of the previous step (0 at the first step of a segment)
  double invnu;      // 1 / nu, nu = ||u - V s|| (reorthogonalised norm)
  double tau_sigma;  // tau * sigma: coefficient of u_raw in the w' update
  double beta_out;   // norm of the residual vector at the end (BVMatArnoldi's *beta)
  double onorm;      // norm before the last pass (for the linear dependence test)
  int stop;          // factorisation ended (breakdown): later kernels of the segment return at once
  int m;             // columns produced (BVMatArnoldi's *m)
  int breakdown;     // BVMatArnoldi's *breakdown
  int k0;            // first column of the segment
  unsigned tickets[8];  // last-block counters, one per kernel kind (reset by the last block)
};

// Epilogue modes of the Gram-Schmidt pair.
enum GSMode : int {
  GS_STEP = 0,    // one DCGS2 Krylov step (NX = 2)
  GS_FINAL = 1,   // final reorthogonalisation of the residual vector (NX = 1)
  GS_ORTHO = 2,   // one CGS pass that orthonormalises u against V (start vectors, BVOrthonormalizeColumn)
  GS_DOTS = 3,    // plain sums: coef[0..J) = sigma V^T u, coef[J] = sigma^2 u.u (BVDotVec, norms)
  GS_COMBINE = 4  // kernel B only: u <- (sigma u - V coef) * invnu, no norm (BVMultVec)
};

// Restart/convergence control written by the projected-problem kernel and read by the host once per restart.
struct KSControl {
  int nconv;        // converged count after this restart (k)
  int l;            // kept (non-converged) vectors
  int reason;       // EPSConvergedReason: 0 iterating, 1 converged, -1 diverged its, -2 breakdown
  int nv;           // size of the projected problem that was solved
  int breakdown;    // the factorisation broke down
  int need_start;   // a new start vector is needed at column nconv (breakdown or k == nv with k < nev)
  int ds_error;     // nonzero if the dense solver did not converge
  int ds_fallback;  // the mixed-precision symmetric solver failed its accuracy check; the FP64 QR solver ran
  double beta;      // residual norm used in the convergence test
  double hgamma;    // harmonic extraction: the scale gamma of the recovered residual vector (work holds g~)
};

// Arguments of one Gram-Schmidt step kernel (both halves of the fused pair).
struct StepArgs {
  const void *V;     // basis, column-major (columns 0..J-1 take part); double or float2 per the storage format
  long long ldv;     // leading dimension (rows, padded)
  int n;             // rows
  int J;             // columns of V taking part (0..J-1)
  int j;             // Krylov index of u (Hessenberg column j); w is the vector of index j+1
  int hermitian;     // 1: write alpha/beta to (d, e); 0: write Hessenberg columns to H
  void *U;           // u (raw, scaled by sigma); overwritten by kernel B with the orthonormal v_j
  void *W;           // w = A u (NX = 2); overwritten by kernel B with w'
  double *d, *e;     // tridiagonal storage (hermitian)
  double *H;         // Hessenberg storage (non-hermitian), column-major ldh
  int ldh;
  double eta;        // linear dependence threshold (0.7071)
  double *coef;      // device scratch for s (coef[0..J)) and g (coef[J..2J))
  float2 *part;      // per-block partial sums
  int pstride;       // stride between blocks in part (float2 units)
  KrylovState *st;
  const GTArgs *tc;  // host side: non-null routes IEEE-double Gram-Schmidt to the tensor-core kernels (k_gs_tc.cu)
  int nc;            // constraint columns (a deflation space) ahead of the basis in V: columns 0..nc-1 take part in
                     // the projections, and coefficient nc + i belongs to Krylov column i
};

}  // namespace ksg
