// api_batch.cu -- EPSGB300SolveBatch: many EPS objects solved together by the batched Krylov-Schur engine.
//
// Every EPS is set up as usual (EPSSetOperators, EPSSetDimensions, ...); the batch solves all of them at once and
// leaves each EPS in the state EPSSolve would: EPSGetConverged, EPSGetEigenpair and friends read the results.
// One restart cycle of every live instance is one CUDA graph launch (k_batch.cu); the host reads a 16-byte status
// per instance after each cycle, hands breakdowns back to the single-problem code, and retires solved instances.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <vector>

#include "batch_types.h"
#include "internal.h"
#include "kernels.h"

using namespace ksg;

namespace {

struct BatchEngine {
  int device = 0;
  cudaStream_t s = nullptr;
  int cap = 0;          // instances
  int slots = 0;        // slots per cycle: max ncv + 1 (steps 0..ncv-1, final pass at nv <= ncv)
  int max_ld = 0;
  int grid_spmv = 0, grid_dot = 0, grid_upd = 0, grid_rst = 0, grid_ds = 0, grid_inst = 0;
  DBuf<BatchInst> inst;
  DBuf<BatchVB> map_spmv, map_dot, map_upd, map_rst;
  DBuf<int> list;
  DBuf<BatchHdr> hdr;
  DBuf<BatchStatus> status;
  BatchStatus *h_status = nullptr;  // pinned
  cudaGraphExec_t exec = nullptr;
  long long launches_per_cycle = 0;

  ~BatchEngine() {
    if (exec) cudaGraphExecDestroy(exec);
    if (h_status) cudaFreeHost(h_status);
    if (s) cudaStreamDestroy(s);
  }
};

// Size buckets of the tuning table: bucket b holds n in [2^(b+9), 2^(b+10)), clamped to [0, BATCH_BUCKETS).
constexpr int BATCH_BUCKETS = 14;
constexpr int GS_TILE_ROWS = 512;  // rows per tile of both Gram-Schmidt kernels
constexpr int SPMV_VB_ROWS = 256;  // rows per pass of one 256-thread SpMV block (one row per thread)

// tiles per virtual block of the Gram-Schmidt kernels, per size bucket (EPSGB300BatchTune measures them)
int g_gs_tpv[BATCH_BUCKETS] = {8, 8, 8, 8, 8, 8, 8, 8, 8, 8, 8, 8, 8, 8};

int batch_bucket(int n) {
  int b = 0;
  while (b + 1 < BATCH_BUCKETS && n >= (1 << (b + 10))) ++b;
  return b;
}

// virtual blocks of instance n in each kernel.  The Gram-Schmidt counts decide the summation partition (and so
// the rounding) of an instance; they depend on n and the tuning table only, never on the rest of the batch.
int batch_gs_vbs(int n, int cap) {
  const int ntiles = (n + GS_TILE_ROWS - 1) / GS_TILE_ROWS;
  const int tpv = g_gs_tpv[batch_bucket(n)];
  int nb = (ntiles + tpv - 1) / tpv;
  return std::max(1, std::min(nb, cap));
}

// work lists of the live instances
PetscErrorCode batch_upload_maps(BatchEngine &B, const std::vector<BatchInst> &hi, const std::vector<int> &live) {
  std::vector<BatchVB> ms, md, mu, mr;
  for (int i : live) {
    const BatchInst &p = hi[i];
    const int ns = std::max(1, std::min(spmv_blocks_for(p.n, p.lanes), (p.n + 8 * SPMV_VB_ROWS - 1) / (8 * SPMV_VB_ROWS)));
    const int nd = batch_gs_vbs(p.n, gs_dot_blocks(p.n)), nu = batch_gs_vbs(p.n, gs_update_blocks(p.n));
    const int nr = std::max(1, std::min(restart_blocks_for(p.n), (p.n + 1023) / 1024));
    for (int b = 0; b < ns; ++b) ms.push_back({i, b, ns, 0});
    for (int b = 0; b < nd; ++b) md.push_back({i, b, nd, 0});
    for (int b = 0; b < nu; ++b) mu.push_back({i, b, nu, 0});
    for (int b = 0; b < nr; ++b) mr.push_back({i, b, nr, 0});
  }
  auto up = [&](DBuf<BatchVB> &d, const std::vector<BatchVB> &h) -> cudaError_t {
    if (h.size() > d.count) {
      cudaError_t e = d.alloc(h.size() + h.size() / 4 + 16);
      if (e != cudaSuccess) return e;
    }
    return h.empty() ? cudaSuccess
                     : cudaMemcpyAsync(d.p, h.data(), h.size() * sizeof(BatchVB), cudaMemcpyHostToDevice, B.s);
  };
  KSG_CUDA(cudaStreamSynchronize(B.s));  // the previous lists may still be read by a running cycle
  KSG_CUDA(up(B.map_spmv, ms));
  KSG_CUDA(up(B.map_dot, md));
  KSG_CUDA(up(B.map_upd, mu));
  KSG_CUDA(up(B.map_rst, mr));
  KSG_CUDA(cudaMemcpyAsync(B.list.p, live.data(), live.size() * sizeof(int), cudaMemcpyHostToDevice, B.s));
  BatchHdr h = {};
  h.n_spmv = (int)ms.size();
  h.n_dot = (int)md.size();
  h.n_upd = (int)mu.size();
  h.n_rst = (int)mr.size();
  h.n_inst = (int)live.size();
  KSG_CUDA(cudaMemcpyAsync(B.hdr.p, &h, sizeof(h), cudaMemcpyHostToDevice, B.s));
  KSG_CUDA(cudaStreamSynchronize(B.s));  // h is on the stack
  return 0;
}

// the launches of one restart cycle, in stream order (captured once into a graph)
PetscErrorCode batch_enqueue_cycle(BatchEngine &B, long long *launches) {
  long long nl = 0;
  cudaStream_t s = B.s;
  KSG_CUDA(launch_batch_begin(B.inst.p, B.list.p, B.hdr.p, B.grid_inst, s));
  KSG_CUDA(launch_batch_dot(B.inst.p, B.map_dot.p, B.hdr.p, -1, B.grid_dot, s));
  KSG_CUDA(launch_batch_update(B.inst.p, B.map_upd.p, B.hdr.p, -1, B.grid_upd, B.max_ld, s));
  KSG_CUDA(launch_batch_start(B.inst.p, B.list.p, B.hdr.p, B.grid_inst, s));
  nl += 4;
  for (int slot = 0; slot < B.slots; ++slot) {
    KSG_CUDA(launch_batch_spmv(B.inst.p, B.map_spmv.p, B.hdr.p, slot, B.grid_spmv, s));
    KSG_CUDA(launch_batch_dot(B.inst.p, B.map_dot.p, B.hdr.p, slot, B.grid_dot, s));
    KSG_CUDA(launch_batch_update(B.inst.p, B.map_upd.p, B.hdr.p, slot, B.grid_upd, B.max_ld, s));
    nl += 3;
  }
  KSG_CUDA(launch_batch_ds_hep(B.inst.p, B.list.p, B.hdr.p, B.grid_ds, B.max_ld, s));
  KSG_CUDA(launch_batch_ds_nhep(B.inst.p, B.list.p, B.hdr.p, B.grid_ds, B.max_ld, s));
  KSG_CUDA(launch_batch_restart(B.inst.p, B.map_rst.p, B.hdr.p, B.grid_rst, B.max_ld, s));
  KSG_CUDA(launch_batch_control(B.inst.p, B.list.p, B.hdr.p, B.status.p, B.grid_inst, s));
  nl += 4;
  KSG_CUDA(cudaMemcpyAsync(B.h_status, B.status.p, sizeof(BatchStatus) * B.cap, cudaMemcpyDeviceToHost, s));
  *launches = nl;
  return 0;
}

PetscErrorCode batch_build_graph(BatchEngine &B) {
  KSG_CUDA(batch_prepare_restart(B.max_ld));
  KSG_CUDA(batch_prepare_ds_hep(B.max_ld));
  cudaGraph_t g = nullptr;
  KSG_CUDA(cudaStreamBeginCapture(B.s, cudaStreamCaptureModeThreadLocal));
  long long nl = 0;
  PetscErrorCode ierr = batch_enqueue_cycle(B, &nl);
  cudaError_t ce = cudaStreamEndCapture(B.s, &g);
  KSG_TRY(ierr);
  KSG_CUDA(ce);
  if (B.exec) cudaGraphExecDestroy(B.exec);
  B.exec = nullptr;
  ce = cudaGraphInstantiate(&B.exec, g, 0);
  cudaGraphDestroy(g);
  KSG_CUDA(ce);
  B.launches_per_cycle = nl;
  return 0;
}

BatchInst make_inst(EPS eps) {
  BatchInst p = {};
  p.n = eps->n;
  p.hermitian = eps->problem == EPS_HEP;
  p.which = eps->which;
  p.nev = eps->nev_e;
  p.ncv = eps->ncv_e;
  p.mpd = eps->mpd_e;
  p.max_it = eps->maxit_e;
  p.lock = eps->lock;
  p.lanes = eps->lanes;
  p.ld = eps->ld;
  p.tol = eps->tol_e;
  p.keep = eps->keep;
  p.opscale = eps->opscale;
  p.rp = eps->A->d_rp.p;
  p.ci = eps->A->d_ci.p;
  p.va2 = eps->A->d_va2.p;
  p.V = reinterpret_cast<float2 *>(eps->V.p);
  p.ldv = eps->ldv;
  p.d = eps->d.p;
  p.e = eps->e.p;
  p.H = eps->H.p;
  p.Q = eps->Q.p;
  p.eigr = eps->eigr.p;
  p.eigi = eps->eigi.p;
  p.errest = eps->errest.p;
  p.coef = eps->coef.p;
  p.work = eps->work.p;
  p.part = eps->part.p;
  p.pstride = eps->pstride;
  p.st = eps->st.p;
  p.ctl = eps->ctl.p;
  p.phase = BP_START;
  return p;
}

}  // namespace

extern "C" PetscErrorCode EPSGB300SolveBatch(PetscInt count, EPS *eps) {
  KSG_CHECK(count >= 0, PETSC_ERR_ARG_OUTOFRANGE, "Negative count");
  if (count == 0) return 0;
  KSG_CHECK(eps, PETSC_ERR_ARG_NULL, "Null EPS array");
  auto t0 = std::chrono::steady_clock::now();
  int device = -1;
  for (int i = 0; i < count; ++i) {
    KSG_CHECK(eps[i], PETSC_ERR_ARG_NULL, "Null EPS at position %d", i);
    KSG_TRY(EPSSetUp(eps[i]));
    KSG_CHECK(eps[i]->storage == STORE_PAIR, PETSC_ERR_SUP,
              "EPSGB300SolveBatch: EPS %d uses EPS_GB300_ARITH_F64; the batched engine runs the pair arithmetic", i);
    KSG_CHECK(eps[i]->ncv_e <= batch_max_columns() - 1, PETSC_ERR_SUP,
              "EPSGB300SolveBatch: ncv = %d exceeds the batched limit %d", eps[i]->ncv_e, batch_max_columns() - 1);
    if (device < 0) device = eps[i]->device;
    KSG_CHECK(eps[i]->device == device, PETSC_ERR_ARG_INCOMP, "EPSGB300SolveBatch: all EPS must use one device");
    for (int j = 0; j < i; ++j) KSG_CHECK(eps[j] != eps[i], PETSC_ERR_ARG_WRONG, "EPS %d appears twice", i);
  }
  KSG_CUDA(cudaSetDevice(device));
  KSG_CUDA(cudaDeviceSynchronize());  // EPSSetUp work on the objects' own streams
  BatchEngine B;
  B.device = device;
  B.cap = (int)count;
  KSG_CUDA(cudaStreamCreateWithFlags(&B.s, cudaStreamNonBlocking));
  const int sms = num_sms();
  B.grid_spmv = sms * 8;
  B.grid_dot = sms;
  B.grid_upd = sms;
  B.grid_rst = sms * 2;
  B.grid_ds = std::min<int>((int)count, sms * 8);
  B.grid_inst = std::min<int>((int)count, sms * 8);
  std::vector<BatchInst> hi(count);
  std::vector<std::vector<double>> rnd(count);
  for (int i = 0; i < count; ++i) {
    EPS e = eps[i];
    hi[i] = make_inst(e);
    B.slots = std::max(B.slots, e->ncv_e + 1);
    B.max_ld = std::max(B.max_ld, e->ld);
    e->solved = 0;
    e->stats = EPSGB300Stats{};
    // start vector in FP64 into column 1, converted to pairs in column 0 (column 1 is rewritten by the first SpMV)
    const double *src;
    if (!e->v0.empty()) src = e->v0.data();
    else {
      rnd[i].resize(e->n);
      ksg_random_fill(rnd[i].data(), e->n, e->seed, 0);
      src = rnd[i].data();
    }
    double *stage = e->V.p + e->ldv;
    KSG_CUDA(cudaMemcpyAsync(stage, src, sizeof(double) * e->n, cudaMemcpyHostToDevice, B.s));
    KSG_CUDA(launch_f64_to_pair(stage, reinterpret_cast<float2 *>(e->V.p), e->n, B.s));
  }
  KSG_CUDA(B.inst.alloc(count));
  KSG_CUDA(B.list.alloc(count));
  KSG_CUDA(B.hdr.alloc(1));
  KSG_CUDA(B.status.alloc(count));
  KSG_CUDA(cudaMallocHost((void **)&B.h_status, sizeof(BatchStatus) * count));
  KSG_CUDA(cudaMemcpyAsync(B.inst.p, hi.data(), sizeof(BatchInst) * count, cudaMemcpyHostToDevice, B.s));
  std::vector<int> live(count);
  for (int i = 0; i < count; ++i) live[i] = i;
  KSG_TRY(batch_upload_maps(B, hi, live));
  KSG_TRY(batch_build_graph(B));
  rnd.clear();
  std::vector<int> phase(count, BP_START);
  long long cycles = 0;
  std::vector<double> er, ei, es;
  while (!live.empty()) {
    KSG_CUDA(cudaGraphLaunch(B.exec, B.s));
    KSG_CUDA(cudaStreamSynchronize(B.s));
    ++cycles;
    std::vector<int> still;
    bool changed = false;
    for (int i : live) {
      const BatchStatus st = B.h_status[i];
      EPS e = eps[i];
      if (st.phase == BP_HOST) {
        // breakdown: a new random start vector at column nconv, as the single-problem loop does
        int bd = 0;
        KSG_TRY(ksg_eps_new_start_vector(e, st.nconv, &bd));
        BatchInst cur;
        KSG_CUDA(cudaMemcpy(&cur, B.inst.p + i, sizeof(BatchInst), cudaMemcpyDeviceToHost));
        if (bd) {
          cur.phase = BP_DONE;
          cur.reason = EPS_DIVERGED_BREAKDOWN;
        } else {
          KSG_CUDA(launch_segment_begin(e->st.p, cur.k0, cur.nv, e->stream));
          cur.phase = BP_ITER;
        }
        KSG_CUDA(cudaStreamSynchronize(e->stream));
        KSG_CUDA(cudaMemcpy(B.inst.p + i, &cur, sizeof(BatchInst), cudaMemcpyHostToDevice));
        if (bd) {
          B.h_status[i].phase = BP_DONE;
          B.h_status[i].reason = EPS_DIVERGED_BREAKDOWN;
        } else {
          still.push_back(i);
          continue;
        }
      }
      const int ph = B.h_status[i].phase;
      if (ph == BP_START || ph == BP_ITER) {
        still.push_back(i);
        continue;
      }
      changed = true;
      BatchInst fin;
      KSG_CUDA(cudaMemcpy(&fin, B.inst.p + i, sizeof(BatchInst), cudaMemcpyDeviceToHost));
      if (ph == BP_FAILED) {
        KSG_CHECK(false, fin.err, "EPSGB300SolveBatch: problem %d failed (%s)", i,
                  fin.err == 77 ? "initial vector is zero or the Krylov segment is empty"
                                : "the projected eigenproblem solver did not converge");
      }
      // retire: eigenvectors of the non-Hermitian Schur form, results into the EPS (EPSSolve's epilogue)
      const int nconv = fin.nconv, ld = e->ld;
      if (!fin.hermitian && nconv > 0) {
        KSG_CUDA(launch_nhep_vectors(e->H.p, ld, nconv, e->X.p, B.s));
        KSG_CUDA(launch_restart(e->V.p, e->ldv, e->n, 0, nconv, 0, nconv, e->X.p, ld, e->arith, B.s, e->storage));
      }
      er.resize(ld);
      ei.resize(ld);
      es.resize(ld);
      KSG_CUDA(cudaMemcpyAsync(er.data(), e->eigr.p, sizeof(double) * ld, cudaMemcpyDeviceToHost, B.s));
      KSG_CUDA(cudaMemcpyAsync(ei.data(), e->eigi.p, sizeof(double) * ld, cudaMemcpyDeviceToHost, B.s));
      KSG_CUDA(cudaMemcpyAsync(es.data(), e->errest.p, sizeof(double) * ld, cudaMemcpyDeviceToHost, B.s));
      KSG_CUDA(cudaStreamSynchronize(B.s));
      KSG_TRY(ksg_eps_assemble(e, nconv, er.data(), ei.data(), es.data(), B.s));
      e->nconv = nconv;
      e->its = fin.its;
      e->reason = fin.reason;
      e->stats.krylov_steps = fin.steps;
      e->stats.restarts = fin.its;
      e->solved = 1;
    }
    if (changed || still.size() != live.size()) {
      live.swap(still);
      if (!live.empty()) KSG_TRY(batch_upload_maps(B, hi, live));
    }
  }
  KSG_CUDA(cudaStreamSynchronize(B.s));
  const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  for (int i = 0; i < count; ++i) {
    eps[i]->stats.solve_seconds = secs;
    eps[i]->stats.kernel_launches = cycles * B.launches_per_cycle;
  }
  return 0;
}

// ---------------------------------------------------------------------------------------------------------------
// Autotuner: tiles per virtual block of the Gram-Schmidt kernels, per size bucket, measured on one restart cycle of
// a GPU-filling batch of 2-D Laplacians (plus a fixed diagonal) of the bucket's middle size.
// ---------------------------------------------------------------------------------------------------------------
extern "C" PetscErrorCode EPSGB300BatchGetTuning(PetscInt *tiles, PetscInt count) {
  KSG_CHECK(tiles, PETSC_ERR_ARG_NULL, "Null argument");
  for (int b = 0; b < count && b < BATCH_BUCKETS; ++b) tiles[b] = g_gs_tpv[b];
  return 0;
}

extern "C" PetscErrorCode EPSGB300BatchSetTuning(const PetscInt *tiles, PetscInt count) {
  KSG_CHECK(tiles, PETSC_ERR_ARG_NULL, "Null argument");
  for (int b = 0; b < count && b < BATCH_BUCKETS; ++b)
    KSG_CHECK(tiles[b] >= 1 && tiles[b] <= 1024, PETSC_ERR_ARG_OUTOFRANGE, "tiles per block %d out of range",
              (int)tiles[b]);
  for (int b = 0; b < count && b < BATCH_BUCKETS; ++b) g_gs_tpv[b] = tiles[b];
  return 0;
}

extern "C" PetscErrorCode EPSGB300BatchTune(PetscInt first_bucket, PetscInt last_bucket) {
  KSG_CHECK(first_bucket >= 0 && last_bucket < BATCH_BUCKETS && first_bucket <= last_bucket,
            PETSC_ERR_ARG_OUTOFRANGE, "buckets must lie in [0, %d]", BATCH_BUCKETS - 1);
  const int cand[] = {1, 2, 4, 8, 16, 32};
  for (int b = (int)first_bucket; b <= (int)last_bucket; ++b) {
    const int nt = 3 << (b + 8);  // middle of [2^(b+9), 2^(b+10))
    const int r = (int)std::sqrt((double)nt), c = (nt + r - 1) / r, n = r * c;
    const int count = std::max(8, std::min(1024, (1 << 23) / n));
    // CSR of the r x c 5-point Laplacian plus diag(0.5 + 0.5 sin(i))
    std::vector<PetscInt> rp(n + 1), ci;
    std::vector<PetscScalar> va;
    ci.reserve(5 * (size_t)n);
    va.reserve(5 * (size_t)n);
    for (int i = 0; i < r; ++i)
      for (int j = 0; j < c; ++j) {
        const int row = i * c + j;
        auto add = [&](int col, double v) { ci.push_back(col); va.push_back(v); };
        if (i > 0) add(row - c, -1.0);
        if (j > 0) add(row - 1, -1.0);
        add(row, 4.0 + 0.5 + 0.5 * std::sin((double)row));
        if (j < c - 1) add(row + 1, -1.0);
        if (i < r - 1) add(row + c, -1.0);
        rp[row + 1] = (PetscInt)ci.size();
      }
    std::vector<double> v0(n);
    for (int i = 0; i < n; ++i) v0[i] = std::sin(0.37 * i + 1.0) + 0.25 * std::cos(1.91 * i);
    std::vector<Mat> mats(count, nullptr);
    std::vector<EPS> eps(count, nullptr);
    std::vector<Vec> vecs(count, nullptr);
    PetscErrorCode ierr = 0;
    for (int k = 0; k < count && !ierr; ++k) {
      ierr = MatCreateSeqAIJWithArrays(0, n, n, rp.data(), ci.data(), va.data(), &mats[k]);
      if (!ierr) ierr = EPSCreate(0, &eps[k]);
      if (!ierr) ierr = EPSSetOperators(eps[k], mats[k], nullptr);
      if (!ierr) ierr = EPSSetProblemType(eps[k], EPS_HEP);
      if (!ierr) ierr = EPSSetDimensions(eps[k], 8, 24, PETSC_DETERMINE);
      if (!ierr) ierr = EPSSetTolerances(eps[k], 1e-10, 1);
      if (!ierr) ierr = EPSSetWhichEigenpairs(eps[k], EPS_LARGEST_MAGNITUDE);
      if (!ierr) ierr = VecCreateSeqWithArray(0, 1, n, v0.data(), &vecs[k]);
      if (!ierr) ierr = EPSSetInitialSpace(eps[k], 1, &vecs[k]);
    }
    int best = g_gs_tpv[b];
    double best_t = 1e30;
    for (int ci_ = 0; ci_ < (int)(sizeof(cand) / sizeof(cand[0])) && !ierr; ++ci_) {
      g_gs_tpv[b] = cand[ci_];
      double t_min = 1e30;
      for (int rep = 0; rep < 3 && !ierr; ++rep) {
        auto t0 = std::chrono::steady_clock::now();
        ierr = EPSGB300SolveBatch(count, eps.data());
        const double t = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        if (rep > 0) t_min = std::min(t_min, t);
      }
      if (t_min < best_t) {
        best_t = t_min;
        best = cand[ci_];
      }
    }
    g_gs_tpv[b] = best;
    for (int k = 0; k < count; ++k) {
      if (eps[k]) EPSDestroy(&eps[k]);
      if (mats[k]) MatDestroy(&mats[k]);
      if (vecs[k]) VecDestroy(&vecs[k]);
    }
    KSG_TRY(ierr);
  }
  return 0;
}
