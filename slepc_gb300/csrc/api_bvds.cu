// api_bvds.cu -- C API: BV (device-resident basis) and DS (projected problem solved on the device).
//
// The BV operations run the same kernels as the eigensolver: BVDotVec is the dot half of the Gram-Schmidt pair,
// BVMultVec its update half, BVMultInPlace the thick-restart kernel, BVMatArnoldi/BVMatLanczos the DCGS2
// factorisation.  DS keeps its matrices on the host between calls (the reference's DSGetArray contract) and
// runs each operation on the device.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "internal.h"

using namespace ksg;

struct _p_BV {
  int n = 0, m = 0;
  int l = 0, k = 0;
  long long ldv = 0;
  int refine = BV_ORTHOG_REFINE_IFNEEDED;
  double eta = 0.7071;
  int arith = ARITH_PAIR;
  cudaStream_t stream = nullptr;
  DBuf<double> V, coef, xvec, yvec;
  DBuf<float2> part;
  DBuf<KrylovState> st;
  int pstride = 0;
  unsigned long long rng = 0;
};

static PetscErrorCode bv_ready(BV bv) {
  KSG_CHECK(bv, PETSC_ERR_ARG_NULL, "Null BV");
  KSG_CHECK(bv->V.p, PETSC_ERR_ORDER, "BVSetSizes must be called first");
  return 0;
}

extern "C" PetscErrorCode BVCreate(MPI_Comm, BV *bv) {
  KSG_CHECK(bv, PETSC_ERR_ARG_NULL, "Null BV pointer");
  *bv = new _p_BV();
  return 0;
}

extern "C" PetscErrorCode BVSetSizes(BV bv, PetscInt n, PetscInt N, PetscInt m) {
  KSG_CHECK(bv, PETSC_ERR_ARG_NULL, "Null BV");
  if (n == PETSC_DECIDE) n = N;
  KSG_CHECK(n > 0 && m > 0, PETSC_ERR_ARG_OUTOFRANGE, "Sizes must be positive");
  KSG_CHECK(N == PETSC_DECIDE || N == n, PETSC_ERR_ARG_SIZ, "Local and global sizes differ on one process");
  KSG_CHECK(m + 1 <= gs_max_columns(), PETSC_ERR_SUP, "At most %d columns", gs_max_columns() - 1);
  bv->n = n;
  bv->m = m;
  bv->l = 0;
  bv->k = m;
  bv->ldv = ((long long)n + 63) / 64 * 64;
  if (!bv->stream) KSG_CUDA(cudaStreamCreateWithFlags(&bv->stream, cudaStreamNonBlocking));
  KSG_CUDA(bv->V.alloc((size_t)bv->ldv * (m + 1)));
  KSG_CUDA(cudaMemset(bv->V.p, 0, sizeof(double) * bv->V.count));
  KSG_CUDA(bv->coef.alloc(2 * (m + 2) + 8));
  KSG_CUDA(bv->xvec.alloc(bv->ldv));
  KSG_CUDA(bv->yvec.alloc(bv->ldv));
  bv->pstride = (int)ksg_part_stride(m + 2);
  KSG_CUDA(bv->part.alloc(ksg_part_blocks(n) * bv->pstride));
  KSG_CUDA(bv->st.alloc(1));
  KSG_CUDA(cudaMemset(bv->st.p, 0, sizeof(KrylovState)));
  return 0;
}

extern "C" PetscErrorCode BVGetSizes(BV bv, PetscInt *n, PetscInt *N, PetscInt *m) {
  KSG_CHECK(bv, PETSC_ERR_ARG_NULL, "Null BV");
  if (n) *n = bv->n;
  if (N) *N = bv->n;
  if (m) *m = bv->m;
  return 0;
}

extern "C" PetscErrorCode BVDestroy(BV *bv) {
  if (!bv || !*bv) return 0;
  if ((*bv)->stream) cudaStreamDestroy((*bv)->stream);
  delete *bv;
  *bv = nullptr;
  return 0;
}

extern "C" PetscErrorCode BVSetActiveColumns(BV bv, PetscInt l, PetscInt k) {
  KSG_TRY(bv_ready(bv));
  KSG_CHECK(k >= 0 && k <= bv->m, PETSC_ERR_ARG_OUTOFRANGE, "Illegal value of k");
  KSG_CHECK(l >= 0 && l <= k, PETSC_ERR_ARG_OUTOFRANGE, "Illegal value of l");
  bv->l = l;
  bv->k = k;
  return 0;
}
extern "C" PetscErrorCode BVGetActiveColumns(BV bv, PetscInt *l, PetscInt *k) {
  KSG_TRY(bv_ready(bv));
  if (l) *l = bv->l;
  if (k) *k = bv->k;
  return 0;
}
extern "C" PetscErrorCode BVSetOrthogonalization(BV bv, BVOrthogType type, BVOrthogRefineType refine, PetscReal eta,
                                                 BVOrthogBlockType) {
  KSG_CHECK(bv, PETSC_ERR_ARG_NULL, "Null BV");
  KSG_CHECK(type == BV_ORTHOG_CGS, PETSC_ERR_SUP, "Only classical Gram-Schmidt is provided");
  bv->refine = refine;
  if (eta != (PetscReal)PETSC_DETERMINE && eta != (PetscReal)PETSC_CURRENT) {
    KSG_CHECK(eta > 0.0 && eta <= 1.0, PETSC_ERR_ARG_OUTOFRANGE, "Invalid eta value");
    bv->eta = eta;
  }
  return 0;
}

static double *bv_col(BV bv, int j) { return bv->V.p + (size_t)j * bv->ldv; }

extern "C" PetscErrorCode BVInsertVec(BV V, PetscInt j, Vec w) {
  KSG_TRY(bv_ready(V));
  KSG_CHECK(w && w->n == V->n, PETSC_ERR_ARG_SIZ, "Vector of the wrong size");
  KSG_CHECK(j >= 0 && j < V->m, PETSC_ERR_ARG_OUTOFRANGE, "Column out of range");
  KSG_CUDA(cudaMemcpy(bv_col(V, j), w->a, sizeof(double) * V->n, cudaMemcpyHostToDevice));
  return 0;
}
extern "C" PetscErrorCode BVCopyVec(BV V, PetscInt j, Vec v) {
  KSG_TRY(bv_ready(V));
  KSG_CHECK(v && v->n == V->n, PETSC_ERR_ARG_SIZ, "Vector of the wrong size");
  KSG_CHECK(j >= 0 && j <= V->m, PETSC_ERR_ARG_OUTOFRANGE, "Column out of range");
  KSG_CUDA(cudaMemcpy(v->a, bv_col(V, j), sizeof(double) * V->n, cudaMemcpyDeviceToHost));
  return 0;
}
extern "C" PetscErrorCode BVCopyColumn(BV V, PetscInt j, PetscInt i) {
  KSG_TRY(bv_ready(V));
  KSG_CHECK(j >= 0 && j <= V->m && i >= 0 && i <= V->m, PETSC_ERR_ARG_OUTOFRANGE, "Column out of range");
  if (i == j) return 0;
  KSG_CUDA(cudaMemcpy(bv_col(V, i), bv_col(V, j), sizeof(double) * V->n, cudaMemcpyDeviceToDevice));
  return 0;
}
extern "C" PetscErrorCode BVScaleColumn(BV bv, PetscInt j, PetscScalar alpha) {
  KSG_TRY(bv_ready(bv));
  KSG_CHECK(j >= 0 && j <= bv->m, PETSC_ERR_ARG_OUTOFRANGE, "Column out of range");
  KSG_CUDA(launch_scale(bv_col(bv, j), bv->n, alpha, bv->stream));
  KSG_CUDA(cudaStreamSynchronize(bv->stream));
  return 0;
}
extern "C" PetscErrorCode BVSetRandomColumn(BV bv, PetscInt j) {
  KSG_TRY(bv_ready(bv));
  KSG_CHECK(j >= 0 && j <= bv->m, PETSC_ERR_ARG_OUTOFRANGE, "Column out of range");
  std::vector<double> h(bv->n);
  ksg_random_fill(h.data(), bv->n, 0xB5EEDULL, ++bv->rng);
  KSG_CUDA(cudaMemcpy(bv_col(bv, j), h.data(), sizeof(double) * bv->n, cudaMemcpyHostToDevice));
  return 0;
}

static StepArgs bv_args(BV bv, int J, double *u) {
  StepArgs a = {};
  a.V = bv->V.p + (size_t)bv->l * bv->ldv;
  a.ldv = bv->ldv;
  a.n = bv->n;
  a.J = J;
  a.j = J;
  a.hermitian = 1;
  a.U = u;
  a.eta = bv->eta;
  a.coef = bv->coef.p;
  a.part = bv->part.p;
  a.pstride = bv->pstride;
  a.st = bv->st.p;
  return a;
}

extern "C" PetscErrorCode BVDotVec(BV X, Vec y, PetscScalar m[]) {
  KSG_TRY(bv_ready(X));
  KSG_CHECK(y && y->n == X->n && m, PETSC_ERR_ARG_SIZ, "Nonconforming arguments");
  const int J = X->k - X->l;
  if (J <= 0) return 0;
  KSG_CUDA(cudaMemcpyAsync(X->xvec.p, y->a, sizeof(double) * X->n, cudaMemcpyHostToDevice, X->stream));
  KSG_CUDA(launch_segment_begin(X->st.p, 0, 0, X->stream));
  StepArgs a = bv_args(X, J, X->xvec.p);
  KSG_CUDA(launch_gs_dot(a, 1, GS_DOTS, X->arith, X->stream));
  KSG_CUDA(cudaMemcpyAsync(m, X->coef.p, sizeof(double) * J, cudaMemcpyDeviceToHost, X->stream));
  KSG_CUDA(cudaStreamSynchronize(X->stream));
  return 0;
}

extern "C" PetscErrorCode BVMultVec(BV X, PetscScalar alpha, PetscScalar beta, Vec y, PetscScalar q[]) {
  KSG_TRY(bv_ready(X));
  KSG_CHECK(y && y->n == X->n, PETSC_ERR_ARG_SIZ, "Nonconforming arguments");
  const int J = X->k - X->l;
  KSG_CHECK(J == 0 || q, PETSC_ERR_ARG_NULL, "Null coefficient array");
  // y <- (beta*y - V*(-alpha q)) * 1, the update half in GS_COMBINE form
  std::vector<double> c(std::max(J, 1));
  for (int i = 0; i < J; ++i) c[i] = -alpha * q[i];
  KSG_CUDA(cudaMemcpyAsync(X->xvec.p, y->a, sizeof(double) * X->n, cudaMemcpyHostToDevice, X->stream));
  if (J > 0) KSG_CUDA(cudaMemcpyAsync(X->coef.p, c.data(), sizeof(double) * J, cudaMemcpyHostToDevice, X->stream));
  KSG_CUDA(launch_set_scales(X->st.p, beta, 1.0, X->stream));
  StepArgs a = bv_args(X, J, X->xvec.p);
  KSG_CUDA(launch_gs_update(a, 1, GS_COMBINE, X->arith, X->stream));
  KSG_CUDA(cudaMemcpyAsync(y->a, X->xvec.p, sizeof(double) * X->n, cudaMemcpyDeviceToHost, X->stream));
  KSG_CUDA(cudaStreamSynchronize(X->stream));
  return 0;
}

extern "C" PetscErrorCode BVMultInPlace(BV V, Mat Q, PetscInt s, PetscInt e) {
  KSG_TRY(bv_ready(V));
  KSG_CHECK(Q && Q->dense, PETSC_ERR_ARG_WRONG, "Q must be a dense Mat");
  KSG_CHECK(s >= V->l && s <= V->m, PETSC_ERR_ARG_OUTOFRANGE, "Argument s has wrong value %d", s);
  KSG_CHECK(e >= V->l && e <= V->m, PETSC_ERR_ARG_OUTOFRANGE, "Argument e has wrong value %d", e);
  KSG_CHECK(Q->m >= V->k, PETSC_ERR_ARG_SIZ, "Mat argument has %d rows, should have at least %d", Q->m, V->k);
  KSG_CHECK(e <= Q->n, PETSC_ERR_ARG_SIZ, "Mat argument only has %d columns", Q->n);
  if (s >= e || V->k <= V->l) return 0;
  DBuf<double> dq;
  KSG_CUDA(dq.alloc((size_t)Q->lda * Q->n));
  KSG_CUDA(cudaMemcpyAsync(dq.p, Q->data, sizeof(double) * Q->lda * Q->n, cudaMemcpyHostToDevice, V->stream));
  KSG_CUDA(launch_restart(V->V.p, V->ldv, V->n, V->l, V->k - V->l, s, e - s, dq.p, Q->lda, V->arith, V->stream));
  KSG_CUDA(cudaStreamSynchronize(V->stream));
  return 0;
}

extern "C" PetscErrorCode BVNormColumn(BV bv, PetscInt j, NormType type, PetscReal *val) {
  KSG_TRY(bv_ready(bv));
  KSG_CHECK(val, PETSC_ERR_ARG_NULL, "Null output");
  KSG_CHECK(j >= 0 && j <= bv->m, PETSC_ERR_ARG_OUTOFRANGE, "Column out of range");
  KSG_CHECK(type == NORM_2 || type == NORM_FROBENIUS, PETSC_ERR_SUP, "Only the 2-norm of a column is provided");
  KSG_CUDA(launch_segment_begin(bv->st.p, 0, 0, bv->stream));
  StepArgs a = bv_args(bv, 0, bv_col(bv, j));
  KSG_CUDA(launch_gs_dot(a, 1, GS_DOTS, bv->arith, bv->stream));
  double h = 0.0;
  KSG_CUDA(cudaMemcpyAsync(&h, bv->coef.p, sizeof(double), cudaMemcpyDeviceToHost, bv->stream));
  KSG_CUDA(cudaStreamSynchronize(bv->stream));
  *val = sqrt(h > 0.0 ? h : 0.0);
  return 0;
}

extern "C" PetscErrorCode BVNorm(BV bv, NormType type, PetscReal *val) {
  KSG_TRY(bv_ready(bv));
  KSG_CHECK(val, PETSC_ERR_ARG_NULL, "Null output");
  KSG_CHECK(type != NORM_2 && type != NORM_1_AND_2, PETSC_ERR_SUP, "Requested norm not available");
  const int l = bv->l, k = bv->k;
  if (type == NORM_FROBENIUS) {
    double s = 0.0;
    for (int j = l; j < k; ++j) {
      double c;
      KSG_TRY(BVNormColumn(bv, j, NORM_2, &c));
      s += c * c;
    }
    *val = sqrt(s);
    return 0;
  }
  // 1- and inf-norms of the active block from a host copy (diagnostic path)
  std::vector<double> h((size_t)bv->n * std::max(k - l, 1));
  for (int j = l; j < k; ++j)
    KSG_CUDA(cudaMemcpy(h.data() + (size_t)(j - l) * bv->n, bv_col(bv, j), sizeof(double) * bv->n, cudaMemcpyDeviceToHost));
  double r = 0.0;
  if (type == NORM_1) {
    for (int j = 0; j < k - l; ++j) {
      double s = 0.0;
      for (int i = 0; i < bv->n; ++i) s += fabs(h[(size_t)j * bv->n + i]);
      r = std::max(r, s);
    }
  } else {
    for (int i = 0; i < bv->n; ++i) {
      double s = 0.0;
      for (int j = 0; j < k - l; ++j) s += fabs(h[(size_t)j * bv->n + i]);
      r = std::max(r, s);
    }
  }
  *val = r;
  return 0;
}

// BVOrthonormalizeColumn (bvorthog.c:380-427): CGS with the BV's refinement, optional random replacement
extern "C" PetscErrorCode BVOrthonormalizeColumn(BV bv, PetscInt j, PetscBool replace, PetscReal *norm, PetscBool *lindep) {
  KSG_TRY(bv_ready(bv));
  KSG_CHECK(j >= 0, PETSC_ERR_ARG_OUTOFRANGE, "Index j must be non-negative");
  KSG_CHECK(j < bv->m, PETSC_ERR_ARG_OUTOFRANGE, "Index j=%d but BV only has %d columns", j, bv->m);
  const int refine = bv->refine == BV_ORTHOG_REFINE_IFNEEDED ? 0 : (bv->refine == BV_ORTHOG_REFINE_NEVER ? 1 : 2);
  double nrm = 0.0;
  int ld = 0;
  KSG_TRY(ksg_orthonormalize_column(bv->V.p, bv->ldv, bv->n, j, bv->coef.p, bv->part.p, bv->pstride, bv->st.p,
                                    bv->arith, bv->stream, &nrm, &ld, refine));
  for (int attempt = 0; replace && (nrm == 0.0 || ld) && attempt < 2; ++attempt) {
    KSG_TRY(BVSetRandomColumn(bv, j));
    KSG_TRY(ksg_orthonormalize_column(bv->V.p, bv->ldv, bv->n, j, bv->coef.p, bv->part.p, bv->pstride, bv->st.p,
                                      bv->arith, bv->stream, &nrm, &ld, refine));
  }
  if (norm) *norm = nrm;
  if (lindep) *lindep = ld ? PETSC_TRUE : PETSC_FALSE;
  return 0;
}

// BVMatArnoldi / BVMatLanczos (bvkrylov.c:56-226) through the DCGS2 step kernels
static PetscErrorCode bv_krylov(BV V, Mat A, Mat H, int herm, PetscInt k, PetscInt *m, PetscReal *beta, PetscBool *breakdown) {
  KSG_TRY(bv_ready(V));
  KSG_CHECK(A && m, PETSC_ERR_ARG_NULL, "Null argument");
  KSG_CHECK(A->m == V->n && A->n == V->n, PETSC_ERR_ARG_SIZ, "Nonconforming operator");
  KSG_CHECK(k >= 0 && k <= V->m, PETSC_ERR_ARG_OUTOFRANGE, "Argument k has wrong value %d", k);
  KSG_CHECK(*m > 0 && *m <= V->m, PETSC_ERR_ARG_OUTOFRANGE, "Argument m has wrong value %d", *m);
  KSG_CHECK(*m > k, PETSC_ERR_ARG_OUTOFRANGE, "Argument m should be at least equal to k+1");
  KSG_TRY(ksg_mat_upload(A));
  const int mm = *m, ld = mm + 2;
  DBuf<double> dH, dd, de;
  KSG_CUDA(dH.alloc((size_t)ld * ld));
  KSG_CUDA(dd.alloc(ld));
  KSG_CUDA(de.alloc(ld));
  KSG_CUDA(cudaMemset(dH.p, 0, sizeof(double) * dH.count));
  KSG_CUDA(cudaMemset(dd.p, 0, sizeof(double) * ld));
  KSG_CUDA(cudaMemset(de.p, 0, sizeof(double) * ld));
  if (H && !herm) {
    KSG_CHECK(H->dense && H->m >= mm && H->n >= mm, PETSC_ERR_ARG_SIZ, "Matrix H too small");
    const int rows = std::min(H->m, ld);
    for (int c = 0; c < std::min(H->n, mm); ++c)
      KSG_CUDA(cudaMemcpy(dH.p + (size_t)c * ld, H->data + (size_t)c * H->lda, sizeof(double) * rows, cudaMemcpyHostToDevice));
  }
  if (H && herm) {
    KSG_CHECK(H->dense && H->m >= mm && H->n >= 2, PETSC_ERR_ARG_SIZ, "Matrix T too small");
    KSG_CUDA(cudaMemcpy(dd.p, H->data, sizeof(double) * mm, cudaMemcpyHostToDevice));
    KSG_CUDA(cudaMemcpy(de.p, H->data + H->lda, sizeof(double) * mm, cudaMemcpyHostToDevice));
  }
  cudaStream_t s = V->stream;
  KSG_CUDA(launch_segment_begin(V->st.p, k, mm, s));
  StepArgs a = {};
  a.V = V->V.p;
  a.ldv = V->ldv;
  a.n = V->n;
  a.hermitian = herm;
  a.d = dd.p;
  a.e = de.p;
  a.H = dH.p;
  a.ldh = ld;
  a.eta = V->eta;
  a.coef = V->coef.p;
  a.part = V->part.p;
  a.pstride = V->pstride;
  a.st = V->st.p;
  const int lanes = spmv_lanes_for((double)A->nnz / A->m);
  for (int j = k; j < mm; ++j) {
    double *u = bv_col(V, j), *w = bv_col(V, j + 1);
    KSG_CUDA(launch_spmv(A->d_rp.p, A->d_ci.p, A->d_va.p, u, w, V->n, lanes, V->st.p, 1.0, s));
    a.J = j;
    a.j = j;
    a.U = u;
    a.W = w;
    KSG_CUDA(launch_gs_dot(a, 2, GS_STEP, V->arith, s));
    KSG_CUDA(launch_gs_update(a, 2, GS_STEP, V->arith, s));
  }
  a.J = mm;
  a.j = mm;
  a.U = bv_col(V, mm);
  a.W = nullptr;
  KSG_CUDA(launch_gs_dot(a, 1, GS_FINAL, V->arith, s));
  KSG_CUDA(launch_gs_update(a, 1, GS_FINAL, V->arith, s));
  KrylovState h;
  KSG_CUDA(cudaMemcpyAsync(&h, V->st.p, sizeof(h), cudaMemcpyDeviceToHost, s));
  KSG_CUDA(cudaStreamSynchronize(s));
  *m = h.m;
  if (beta) *beta = h.beta_out;
  if (breakdown) *breakdown = h.breakdown ? PETSC_TRUE : PETSC_FALSE;
  if (H && !herm) {
    for (int c = k; c < h.m; ++c) {
      const int rows = std::min(c + 2, H->m);
      KSG_CUDA(cudaMemcpy(H->data + (size_t)c * H->lda, dH.p + (size_t)c * ld, sizeof(double) * rows, cudaMemcpyDeviceToHost));
    }
  }
  if (H && herm) {
    std::vector<double> hd(ld), he(ld);
    KSG_CUDA(cudaMemcpy(hd.data(), dd.p, sizeof(double) * ld, cudaMemcpyDeviceToHost));
    KSG_CUDA(cudaMemcpy(he.data(), de.p, sizeof(double) * ld, cudaMemcpyDeviceToHost));
    for (int c = k; c < h.m; ++c) {
      H->data[c] = hd[c];
      H->data[H->lda + c] = he[c];
    }
  }
  return 0;
}

extern "C" PetscErrorCode BVMatArnoldi(BV V, Mat A, Mat H, PetscInt k, PetscInt *m, PetscReal *beta, PetscBool *breakdown) {
  return bv_krylov(V, A, H, 0, k, m, beta, breakdown);
}
extern "C" PetscErrorCode BVMatLanczos(BV V, Mat A, Mat T, PetscInt k, PetscInt *m, PetscReal *beta, PetscBool *breakdown) {
  return bv_krylov(V, A, T, 1, k, m, beta, breakdown);
}

// ---------------------------------------------------------------------------------------------------------------
// DS
// ---------------------------------------------------------------------------------------------------------------
struct _p_DS {
  int type = 0;  // 1 hep, 2 nhep
  int ld = 0, n = 0, l = 0, k = 0, t = 0;
  int state = DS_STATE_RAW;
  int compact = 0, extrarow = 0;
  std::vector<double> A, Q, X, T;  // T: 3 columns of ld (d, e, unused)
  std::vector<double> wr, wi;
  struct _n_SlepcSC sc = {};
  int which = 0;
};

extern "C" PetscErrorCode SlepcCompareLargestMagnitude(PetscScalar ar, PetscScalar ai, PetscScalar br, PetscScalar bi, PetscInt *r, void *) {
  const double a = hypot(ar, ai), b = hypot(br, bi);
  *r = a < b ? 1 : (a > b ? -1 : 0);
  return 0;
}
extern "C" PetscErrorCode SlepcCompareSmallestMagnitude(PetscScalar ar, PetscScalar ai, PetscScalar br, PetscScalar bi, PetscInt *r, void *) {
  const double a = hypot(ar, ai), b = hypot(br, bi);
  *r = a > b ? 1 : (a < b ? -1 : 0);
  return 0;
}
extern "C" PetscErrorCode SlepcCompareLargestReal(PetscScalar ar, PetscScalar, PetscScalar br, PetscScalar, PetscInt *r, void *) {
  *r = ar < br ? 1 : (ar > br ? -1 : 0);
  return 0;
}
extern "C" PetscErrorCode SlepcCompareSmallestReal(PetscScalar ar, PetscScalar, PetscScalar br, PetscScalar, PetscInt *r, void *) {
  *r = ar > br ? 1 : (ar < br ? -1 : 0);
  return 0;
}
extern "C" PetscErrorCode SlepcCompareLargestImaginary(PetscScalar, PetscScalar ai, PetscScalar, PetscScalar bi, PetscInt *r, void *) {
  const double a = fabs(ai), b = fabs(bi);
  *r = a < b ? 1 : (a > b ? -1 : 0);
  return 0;
}
extern "C" PetscErrorCode SlepcCompareSmallestImaginary(PetscScalar, PetscScalar ai, PetscScalar, PetscScalar bi, PetscInt *r, void *) {
  const double a = fabs(ai), b = fabs(bi);
  *r = a > b ? 1 : (a < b ? -1 : 0);
  return 0;
}

static int ds_which_of(DS ds) {
  const SlepcSCCompareFn f = ds->sc.comparison;
  if (f == SlepcCompareLargestMagnitude) return 1;
  if (f == SlepcCompareSmallestMagnitude) return 2;
  if (f == SlepcCompareLargestReal) return 3;
  if (f == SlepcCompareSmallestReal) return 4;
  if (f == SlepcCompareLargestImaginary) return 5;
  if (f == SlepcCompareSmallestImaginary) return 6;
  return 0;
}

extern "C" PetscErrorCode DSCreate(MPI_Comm, DS *ds) {
  KSG_CHECK(ds, PETSC_ERR_ARG_NULL, "Null DS pointer");
  *ds = new _p_DS();
  return 0;
}
extern "C" PetscErrorCode DSSetType(DS ds, DSType type) {
  KSG_CHECK(ds && type, PETSC_ERR_ARG_NULL, "Null argument");
  if (!strcmp(type, DSHEP)) ds->type = 1;
  else if (!strcmp(type, DSNHEP)) ds->type = 2;
  else return ksg_set_error(PETSC_ERR_SUP, "Only DSHEP and DSNHEP are provided");
  return 0;
}
extern "C" PetscErrorCode DSAllocate(DS ds, PetscInt ld) {
  KSG_CHECK(ds, PETSC_ERR_ARG_NULL, "Null DS");
  KSG_CHECK(ds->type, PETSC_ERR_ORDER, "Must call DSSetType() first");
  KSG_CHECK(ld > 0 && ld <= KSG_HOST_DS_MAX_LD, PETSC_ERR_ARG_OUTOFRANGE, "Leading dimension must be in 1..%d",
            KSG_HOST_DS_MAX_LD);
  ds->ld = ld;
  ds->A.assign((size_t)ld * ld, 0.0);
  ds->Q.assign((size_t)ld * ld, 0.0);
  ds->X.assign((size_t)ld * ld, 0.0);
  ds->T.assign((size_t)3 * ld, 0.0);
  ds->wr.assign(ld, 0.0);
  ds->wi.assign(ld, 0.0);
  ds->n = ds->t = ld;
  return 0;
}
extern "C" PetscErrorCode DSGetLeadingDimension(DS ds, PetscInt *ld) {
  KSG_CHECK(ds && ld, PETSC_ERR_ARG_NULL, "Null argument");
  *ld = ds->ld;
  return 0;
}
extern "C" PetscErrorCode DSSetDimensions(DS ds, PetscInt n, PetscInt l, PetscInt k) {
  KSG_CHECK(ds, PETSC_ERR_ARG_NULL, "Null DS");
  KSG_CHECK(ds->ld, PETSC_ERR_ORDER, "Must call DSAllocate() first");
  if (n == PETSC_DETERMINE) n = ds->extrarow ? ds->ld - 1 : ds->ld;
  if (n != PETSC_CURRENT) {
    KSG_CHECK(n >= 0 && n <= ds->ld, PETSC_ERR_ARG_OUTOFRANGE, "Illegal value of n. Must be between 0 and ld");
    KSG_CHECK(!ds->extrarow || n < ds->ld, PETSC_ERR_ARG_OUTOFRANGE, "A value of n equal to ld leaves no room for extra row");
    ds->n = n;
  }
  ds->t = ds->n;
  if (l == PETSC_DETERMINE) ds->l = 0;
  else if (l != PETSC_CURRENT) {
    KSG_CHECK(l >= 0 && l <= ds->n, PETSC_ERR_ARG_OUTOFRANGE, "Illegal value of l. Must be between 0 and n");
    ds->l = l;
  }
  if (k == PETSC_DETERMINE) ds->k = ds->n / 2;
  else if (k != PETSC_CURRENT) ds->k = k;
  return 0;
}
extern "C" PetscErrorCode DSGetDimensions(DS ds, PetscInt *n, PetscInt *l, PetscInt *k, PetscInt *t) {
  KSG_CHECK(ds, PETSC_ERR_ARG_NULL, "Null DS");
  if (n) *n = ds->n;
  if (l) *l = ds->l;
  if (k) *k = ds->k;
  if (t) *t = ds->t;
  return 0;
}
extern "C" PetscErrorCode DSSetState(DS ds, DSStateType state) {
  KSG_CHECK(ds, PETSC_ERR_ARG_NULL, "Null DS");
  ds->state = state;
  return 0;
}
extern "C" PetscErrorCode DSGetState(DS ds, DSStateType *state) {
  KSG_CHECK(ds && state, PETSC_ERR_ARG_NULL, "Null argument");
  *state = (DSStateType)ds->state;
  return 0;
}
extern "C" PetscErrorCode DSSetCompact(DS ds, PetscBool comp) {
  KSG_CHECK(ds, PETSC_ERR_ARG_NULL, "Null DS");
  ds->compact = comp ? 1 : 0;
  return 0;
}
extern "C" PetscErrorCode DSSetExtraRow(DS ds, PetscBool ext) {
  KSG_CHECK(ds, PETSC_ERR_ARG_NULL, "Null DS");
  KSG_CHECK(!(ds->ld && ext && ds->n == ds->ld), PETSC_ERR_ARG_OUTOFRANGE, "Cannot set extra row after setting n=ld");
  ds->extrarow = ext ? 1 : 0;
  return 0;
}
extern "C" PetscErrorCode DSGetSlepcSC(DS ds, SlepcSC *sc) {
  KSG_CHECK(ds && sc, PETSC_ERR_ARG_NULL, "Null argument");
  *sc = &ds->sc;
  return 0;
}
extern "C" PetscErrorCode DSGetArray(DS ds, DSMatType m, PetscScalar *a[]) {
  KSG_CHECK(ds && a, PETSC_ERR_ARG_NULL, "Null argument");
  KSG_CHECK(ds->ld, PETSC_ERR_ORDER, "Must call DSAllocate() first");
  switch (m) {
    case DS_MAT_A: *a = ds->A.data(); break;
    case DS_MAT_Q: *a = ds->Q.data(); break;
    case DS_MAT_X: *a = ds->X.data(); break;
    case DS_MAT_T: *a = ds->T.data(); break;
    default: return ksg_set_error(PETSC_ERR_SUP, "Matrix not provided by this DS");
  }
  return 0;
}
extern "C" PetscErrorCode DSRestoreArray(DS, DSMatType, PetscScalar *a[]) {
  if (a) *a = nullptr;
  return 0;
}
extern "C" PetscErrorCode DSGetArrayReal(DS ds, DSMatType m, PetscReal *a[]) {
  KSG_CHECK(m == DS_MAT_T || m == DS_MAT_D, PETSC_ERR_ARG_WRONG, "Only the real matrices T and D");
  return DSGetArray(ds, DS_MAT_T, a);
}
extern "C" PetscErrorCode DSRestoreArrayReal(DS ds, DSMatType m, PetscReal *a[]) { return DSRestoreArray(ds, m, a); }
extern "C" PetscErrorCode DSDestroy(DS *ds) {
  if (!ds || !*ds) return 0;
  delete *ds;
  *ds = nullptr;
  return 0;
}

// run device DS operations on the host-held matrices
static PetscErrorCode ds_run(DS ds, int flags, PetscScalar eigr[], PetscScalar eigi[]) {
  const int ld = ds->ld, n = ds->n;
  DBuf<double> dA, dQ, dd, de, der, dei, des, dw;
  DBuf<KSControl> dc;
  KSG_CUDA(dA.alloc((size_t)ld * ld));
  KSG_CUDA(dQ.alloc((size_t)ld * ld));
  KSG_CUDA(dd.alloc(ld));
  KSG_CUDA(de.alloc(ld));
  KSG_CUDA(der.alloc(ld));
  KSG_CUDA(dei.alloc(ld));
  KSG_CUDA(des.alloc(ld));
  KSG_CUDA(dw.alloc(4 * ld));
  KSG_CUDA(dc.alloc(1));
  KSG_CUDA(cudaMemset(dc.p, 0, sizeof(KSControl)));
  KSG_CUDA(cudaMemcpy(dA.p, ds->A.data(), sizeof(double) * ld * ld, cudaMemcpyHostToDevice));
  KSG_CUDA(cudaMemcpy(dQ.p, ds->Q.data(), sizeof(double) * ld * ld, cudaMemcpyHostToDevice));
  KSG_CUDA(cudaMemcpy(dd.p, ds->T.data(), sizeof(double) * ld, cudaMemcpyHostToDevice));
  KSG_CUDA(cudaMemcpy(de.p, ds->T.data() + ld, sizeof(double) * ld, cudaMemcpyHostToDevice));
  DSArgs a = {};
  a.ld = ld;
  a.n = n;
  a.flags = flags;
  a.l = ds->l;
  a.k = ds->k;
  a.raw = ds->state < DS_STATE_INTERMEDIATE;
  a.d = dd.p;
  a.e = de.p;
  a.H = dA.p;
  a.Q = dQ.p;
  a.eigr = der.p;
  a.eigi = dei.p;
  a.errest = des.p;
  a.work = dw.p;
  a.which = ds->which;
  a.st = nullptr;
  a.ctl = dc.p;
  if (ds->type == 1) {
    KSG_CHECK(ds->compact, PETSC_ERR_SUP, "DSHEP is provided in compact storage only");
    KSG_CUDA(launch_ds_hep(a, n, 0));
  } else {
    KSG_CUDA(launch_ds_nhep(a, n, 0));
  }
  KSControl c;
  KSG_CUDA(cudaMemcpy(&c, dc.p, sizeof(c), cudaMemcpyDeviceToHost));
  KSG_CHECK(!c.ds_error, PETSC_ERR_LIB, "The device dense solver failed (code %d)", c.ds_error);
  KSG_CUDA(cudaMemcpy(ds->A.data(), dA.p, sizeof(double) * ld * ld, cudaMemcpyDeviceToHost));
  KSG_CUDA(cudaMemcpy(ds->Q.data(), dQ.p, sizeof(double) * ld * ld, cudaMemcpyDeviceToHost));
  KSG_CUDA(cudaMemcpy(ds->T.data(), dd.p, sizeof(double) * ld, cudaMemcpyDeviceToHost));
  KSG_CUDA(cudaMemcpy(ds->T.data() + ld, de.p, sizeof(double) * ld, cudaMemcpyDeviceToHost));
  KSG_CUDA(cudaMemcpy(ds->wr.data(), der.p, sizeof(double) * ld, cudaMemcpyDeviceToHost));
  KSG_CUDA(cudaMemcpy(ds->wi.data(), dei.p, sizeof(double) * ld, cudaMemcpyDeviceToHost));
  if (eigr)
    for (int i = 0; i < n; ++i) eigr[i] = ds->wr[i];
  if (eigi)
    for (int i = 0; i < n; ++i) eigi[i] = ds->type == 1 ? 0.0 : ds->wi[i];
  return 0;
}

extern "C" PetscErrorCode DSSolve(DS ds, PetscScalar eigr[], PetscScalar eigi[]) {
  KSG_CHECK(ds && eigr, PETSC_ERR_ARG_NULL, "Null argument");
  KSG_CHECK(ds->ld, PETSC_ERR_ORDER, "Must call DSAllocate() first");
  KSG_CHECK(ds->type == 1 || eigi, PETSC_ERR_ARG_NULL, "eigi is required for DSNHEP");
  if (ds->state >= DS_STATE_CONDENSED) return 0;
  if (ds->type == 2 && ds->n == 1) {
    ds->Q.assign(ds->Q.size(), 0.0);
    ds->Q[0] = 1.0;
    eigr[0] = ds->A[0];
    if (eigi) eigi[0] = 0.0;
    ds->state = DS_STATE_CONDENSED;
    return 0;
  }
  ds->which = ds_which_of(ds);
  KSG_TRY(ds_run(ds, DS_DO_SOLVE, eigr, eigi));
  ds->state = DS_STATE_CONDENSED;
  return 0;
}

extern "C" PetscErrorCode DSSort(DS ds, PetscScalar eigr[], PetscScalar eigi[], PetscScalar rr[], PetscScalar ri[], PetscInt *k) {
  KSG_CHECK(ds && eigr, PETSC_ERR_ARG_NULL, "Null argument");
  KSG_CHECK(!rr && !ri && !k, PETSC_ERR_SUP, "Arbitrary selection is not provided");
  KSG_CHECK(ds->state == DS_STATE_CONDENSED, PETSC_ERR_ORDER, "Must call DSSolve() first");
  ds->which = ds_which_of(ds);
  KSG_CHECK(ds->which, PETSC_ERR_ORDER, "Must provide a sorting criterion first");
  KSG_TRY(ds_run(ds, DS_DO_SORT, eigr, eigi));
  return 0;
}

extern "C" PetscErrorCode DSUpdateExtraRow(DS ds) {
  KSG_CHECK(ds, PETSC_ERR_ARG_NULL, "Null DS");
  KSG_CHECK(ds->extrarow, PETSC_ERR_ARG_WRONGSTATE, "Should have called DSSetExtraRow");
  KSG_CHECK(ds->state >= DS_STATE_CONDENSED, PETSC_ERR_ORDER, "Must call DSSolve() first");
  KSG_TRY(ds_run(ds, DS_DO_EXTRAROW, nullptr, nullptr));
  ds->k = ds->n;
  return 0;
}

extern "C" PetscErrorCode DSTruncate(DS ds, PetscInt n, PetscBool trim) {
  KSG_CHECK(ds, PETSC_ERR_ARG_NULL, "Null DS");
  KSG_CHECK(n >= ds->l && n <= ds->n, PETSC_ERR_ARG_OUTOFRANGE, "Illegal value of n (%d)", n);
  const int ld = ds->ld, l = ds->l;
  if (ds->type == 2 && ds->extrarow) {
    if (trim) {
      for (int i = l; i < ds->n; ++i) ds->A[ds->n + (size_t)i * ld] = 0.0;
    } else if (ds->k == ds->n) {
      for (int i = l; i < n; ++i) ds->A[n + (size_t)i * ld] = ds->A[ds->n + (size_t)i * ld];
      for (int i = l; i < ds->n; ++i) ds->A[ds->n + (size_t)i * ld] = 0.0;
    }
  }
  if (trim) {
    ds->l = 0;
    ds->k = 0;
    ds->n = n;
    ds->t = n;
    ds->state = DS_STATE_RAW;
  } else {
    ds->k = ds->extrarow ? n : 0;
    ds->t = ds->n;
    ds->n = n;
    ds->state = DS_STATE_TRUNCATED;
  }
  return 0;
}

extern "C" PetscErrorCode DSVectors(DS ds, DSMatType mat, PetscInt *j, PetscReal *rnorm) {
  KSG_CHECK(ds, PETSC_ERR_ARG_NULL, "Null DS");
  KSG_CHECK(mat == DS_MAT_X, PETSC_ERR_SUP, "Only DS_MAT_X is provided");
  const int ld = ds->ld, n = ds->n;
  if (ds->type == 1) {
    // DSVectors_HEP (dshep.c:137-172): the eigenvectors are the columns of Q
    if (j) {
      if (ds->state >= DS_STATE_CONDENSED) {
        for (int i = 0; i < ld; ++i) ds->X[i + (size_t)(*j) * ld] = ds->Q[i + (size_t)(*j) * ld];
        if (rnorm) *rnorm = fabs(ds->Q[n - 1 + (size_t)(*j) * ld]);
      } else {
        for (int i = 0; i < ld; ++i) ds->X[i + (size_t)(*j) * ld] = (i == *j) ? 1.0 : 0.0;
        if (rnorm) *rnorm = 0.0;
      }
    } else {
      ds->X = ds->Q;
    }
    return 0;
  }
  // DSNHEP: eigenvectors of T on the device, back-transformed with Q when condensed
  DBuf<double> dA, dX;
  KSG_CUDA(dA.alloc((size_t)ld * ld));
  KSG_CUDA(dX.alloc((size_t)ld * ld));
  KSG_CUDA(cudaMemcpy(dA.p, ds->A.data(), sizeof(double) * ld * ld, cudaMemcpyHostToDevice));
  KSG_CUDA(cudaMemset(dX.p, 0, sizeof(double) * ld * ld));
  KSG_CUDA(launch_nhep_vectors(dA.p, ld, n, dX.p, 0));
  std::vector<double> Y((size_t)ld * ld);
  KSG_CUDA(cudaMemcpy(Y.data(), dX.p, sizeof(double) * ld * ld, cudaMemcpyDeviceToHost));
  auto backtransform = [&](int c, int cols) {
    // columns c (.. c+cols-1) of Y -> Q * Y, normalised jointly (dsnhep.c:101-166)
    double nrm = 0.0;
    std::vector<double> out((size_t)cols * n);
    for (int q = 0; q < cols; ++q)
      for (int i = 0; i < n; ++i) {
        double s = 0.0;
        if (ds->state >= DS_STATE_CONDENSED)
          for (int k2 = 0; k2 < n; ++k2) s += ds->Q[i + (size_t)k2 * ld] * Y[k2 + (size_t)(c + q) * ld];
        else s = Y[i + (size_t)(c + q) * ld];
        out[(size_t)q * n + i] = s;
        nrm += s * s;
      }
    nrm = sqrt(nrm);
    for (int q = 0; q < cols; ++q)
      for (int i = 0; i < n; ++i) ds->X[i + (size_t)(c + q) * ld] = out[(size_t)q * n + i] / nrm;
  };
  if (j) {
    const int c = *j;
    const int cplx = (c < n - 1 && ds->A[c + 1 + (size_t)c * ld] != 0.0);
    backtransform(c, cplx ? 2 : 1);
    if (rnorm) {
      const double yr = ds->X[n - 1 + (size_t)c * ld];
      *rnorm = cplx ? hypot(yr, ds->X[n - 1 + (size_t)(c + 1) * ld]) : fabs(yr);
    }
    if (cplx) (*j)++;
  } else {
    for (int c = 0; c < n; ++c) {
      const int cplx = (c < n - 1 && ds->A[c + 1 + (size_t)c * ld] != 0.0);
      backtransform(c, cplx ? 2 : 1);
      if (cplx) c++;
    }
  }
  return 0;
}

extern "C" PetscErrorCode EPSGetBV(EPS eps, BV *V) {
  KSG_CHECK(eps && V, PETSC_ERR_ARG_NULL, "Null argument");
  KSG_CHECK(eps->setup, PETSC_ERR_ORDER, "Must call EPSSetUp() first");
  if (!eps->bv) {
    KSG_TRY(BVCreate(0, &eps->bv));
    KSG_TRY(BVSetSizes(eps->bv, eps->n, eps->n, eps->ncv_e + 1));
  }
  // expose the solver's basis: copy (or convert from pairs) into the BV, which owns FP64 storage
  if (eps->storage == STORE_PAIR)
    KSG_CUDA(launch_pair_to_f64(reinterpret_cast<const float2 *>(eps->V.p), eps->bv->V.p, eps->ldv * (eps->ncv_e + 1), 0));
  else
    KSG_CUDA(cudaMemcpy(eps->bv->V.p, eps->V.p, sizeof(double) * eps->ldv * (eps->ncv_e + 1), cudaMemcpyDeviceToDevice));
  KSG_CUDA(cudaDeviceSynchronize());
  eps->bv->l = 0;
  eps->bv->k = eps->solved ? eps->nconv : eps->ncv_e;
  *V = eps->bv;
  return 0;
}

extern "C" PetscErrorCode EPSGetDS(EPS eps, DS *ds) {
  KSG_CHECK(eps && ds, PETSC_ERR_ARG_NULL, "Null argument");
  if (!eps->ds) {
    KSG_TRY(DSCreate(0, &eps->ds));  // typed by EPSSetFromOptions (DSNHEP) or EPSSetUp, as the reference's
    if (eps->setup) {
      KSG_TRY(DSSetType(eps->ds, ksg_eps_lanczos(eps) ? DSHEP : DSNHEP));
      if (eps->ld <= KSG_HOST_DS_MAX_LD) KSG_TRY(DSAllocate(eps->ds, eps->ld));
    }
  }
  *ds = eps->ds;
  return 0;
}

extern "C" PetscErrorCode DSGetType(DS ds, DSType *type) {
  KSG_CHECK(ds && type, PETSC_ERR_ARG_NULL, "Null argument");
  *type = ds->type == 1 ? DSHEP : ds->type == 2 ? DSNHEP : nullptr;
  return 0;
}

// DSView, ASCII: "DS Object: 1 MPI process" and the type
extern "C" PetscErrorCode DSView(DS ds, PetscViewer viewer) {
  KSG_CHECK(ds, PETSC_ERR_ARG_NULL, "Null DS");
  if (!viewer) KSG_TRY(PetscViewerASCIIGetStdout(PETSC_COMM_SELF, &viewer));
  if (!viewer->ascii) return 0;
  KSG_TRY(PetscViewerASCIIPrintf(viewer, "DS Object: 1 MPI process\n  %s\n",
                                 ds->type == 1 ? "type: hep" : ds->type == 2 ? "type: nhep" : "type not yet set"));
  return 0;
}
