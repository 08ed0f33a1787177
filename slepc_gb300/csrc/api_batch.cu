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

#include "batch_engine.h"
#include "batch_types.h"
#include "internal.h"
#include "kernels.h"

namespace ksg {

// Size buckets of the tuning table: bucket b holds n in [2^(b+9), 2^(b+10)), clamped to [0, BATCH_BUCKETS).
constexpr int BATCH_BUCKETS = 14;
constexpr int GS_TILE_ROWS = 512;  // rows per tile of both Gram-Schmidt kernels
constexpr int SPMV_VB_ROWS = 256;  // rows per pass of one 256-thread SpMV block (one row per thread)

// tiles per virtual block of the Gram-Schmidt kernels, per size bucket (EPSGB300BatchTune measures them)
static int g_gs_tpv[BATCH_BUCKETS] = {8, 8, 8, 8, 8, 8, 8, 8, 8, 8, 8, 8, 8, 8};

static int batch_bucket(int n) {
  int b = 0;
  while (b + 1 < BATCH_BUCKETS && n >= (1 << (b + 10))) ++b;
  return b;
}

// Virtual blocks of an instance of n rows.  The Gram-Schmidt counts decide the summation partition (and so the
// rounding) of an instance; they depend on n and the tuning table only, never on the rest of the batch.
static int batch_gs_vbs(int n, int cap) {
  const int ntiles = (n + GS_TILE_ROWS - 1) / GS_TILE_ROWS;
  const int tpv = g_gs_tpv[batch_bucket(n)];
  const int nb = (ntiles + tpv - 1) / tpv;
  return std::max(1, std::min(nb, cap));
}

BatchEngine::~BatchEngine() {
  if (exec) cudaGraphExecDestroy(exec);
  if (h_status) cudaFreeHost(h_status);
  if (s) cudaStreamDestroy(s);
}

static BatchInst make_inst(EPS eps) {
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
  p.va32 = eps->A->d_va32.p;
  p.storage = eps->storage;
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

PetscErrorCode ksg_engine_check(EPS e, int max_ncv, bool allow_f32) {
  KSG_CHECK(e->arith == ARITH_PAIR || (allow_f32 && e->arith == ARITH_F32), PETSC_ERR_SUP,
            "batched engine: the EPS must use the pair arithmetic%s", allow_f32 ? " or the precision form" : "");
  KSG_CHECK(e->ncv_e <= max_ncv, PETSC_ERR_SUP, "batched engine: ncv = %d exceeds the limit %d", e->ncv_e, max_ncv);
  KSG_CHECK(e->extraction == EPS_RITZ && e->which <= EPS_SMALLEST_IMAGINARY, PETSC_ERR_SUP,
            "batched engine: Ritz extraction with the largest/smallest criteria only (use EPSSolve for targets)");
  KSG_CHECK(!e->B && e->conv == EPS_CONV_REL, PETSC_ERR_SUP,
            "batched engine: standard problems with the relative convergence test only (use EPSSolve)");
  KSG_CHECK(e->ndefl == 0, PETSC_ERR_SUP, "batched engine: no deflation spaces (use EPSSolve)");
  return 0;
}

PetscErrorCode ksg_engine_init(BatchEngine &B, int device, int cap, int max_ncv, bool with_f32) {
  KSG_CHECK(max_ncv >= 1 && max_ncv <= batch_max_columns() - 1, PETSC_ERR_ARG_OUTOFRANGE,
            "batched engine: ncv limit %d outside [1, %d]", max_ncv, batch_max_columns() - 1);
  B.device = device;
  B.cap = cap;
  B.has_f32 = with_f32;
  B.slots = max_ncv + 1;
  B.max_ld = max_ncv + 1;
  KSG_CUDA(cudaSetDevice(device));
  KSG_CUDA(prepare_ds_nhep());
  KSG_CUDA(cudaStreamCreateWithFlags(&B.s, cudaStreamNonBlocking));
  const int sms = num_sms();
  B.grid_spmv = sms * 8;
  B.grid_dot = sms;
  B.grid_upd = sms;
  B.grid_rst = sms * 2;
  B.grid_ds = std::min(cap, sms * 8);
  B.grid_inst = std::min(cap, sms * 8);
  KSG_CUDA(B.inst.alloc(cap));
  KSG_CUDA(B.list.alloc(cap));
  KSG_CUDA(B.hdr.alloc(1));
  KSG_CUDA(B.status.alloc(cap));
  KSG_CUDA(cudaMallocHost((void **)&B.h_status, sizeof(BatchStatus) * cap));
  BatchHdr h = {};
  KSG_CUDA(cudaMemcpy(B.hdr.p, &h, sizeof(h), cudaMemcpyHostToDevice));
  B.hi.assign(cap, BatchInst{});
  B.eps.assign(cap, nullptr);
  B.free_slots.clear();
  for (int i = cap - 1; i >= 0; --i) B.free_slots.push_back(i);
  return 0;
}

// the launches of one restart cycle, in stream order (captured into a graph)
static PetscErrorCode engine_enqueue_cycle(BatchEngine &B, long long *launches) {
  long long nl = 0;
  cudaStream_t s = B.s;
  KSG_CUDA(launch_batch_begin(B.inst.p, B.list.p, B.hdr.p, B.grid_inst, s));
  for (int q = 0; q < (B.has_f32 ? 2 : 1); ++q) {
    const int st = q ? STORE_F32 : STORE_PAIR;
    KSG_CUDA(launch_batch_dot(B.inst.p, B.map_dot.p, B.hdr.p, -1, B.grid_dot, s, st, B.max_ld));
    KSG_CUDA(launch_batch_update(B.inst.p, B.map_upd.p, B.hdr.p, -1, B.grid_upd, B.max_ld, s, st));
    nl += 2;
  }
  KSG_CUDA(launch_batch_start(B.inst.p, B.list.p, B.hdr.p, B.grid_inst, s));
  nl += 2;
  // the FP32 kernels are captured only when the engine holds precision-form instances
  const int nsto = B.has_f32 ? 2 : 1;
  const int sto[2] = {STORE_PAIR, STORE_F32};
  for (int slot = 0; slot < B.slots; ++slot) {
    for (int q = 0; q < nsto; ++q) {
      KSG_CUDA(launch_batch_spmv(B.inst.p, B.map_spmv.p, B.hdr.p, slot, B.grid_spmv, s, sto[q]));
      KSG_CUDA(launch_batch_dot(B.inst.p, B.map_dot.p, B.hdr.p, slot, B.grid_dot, s, sto[q], B.max_ld));
      KSG_CUDA(launch_batch_update(B.inst.p, B.map_upd.p, B.hdr.p, slot, B.grid_upd, B.max_ld, s, sto[q]));
      nl += 3;
    }
  }
  KSG_CUDA(launch_batch_ds_hep(B.inst.p, B.list.p, B.hdr.p, B.grid_ds, B.max_ld, s));
  KSG_CUDA(launch_batch_ds_nhep(B.inst.p, B.list.p, B.hdr.p, B.grid_ds, B.max_ld, s));
  for (int q = 0; q < nsto; ++q)
    KSG_CUDA(launch_batch_restart(B.inst.p, B.map_rst.p, B.hdr.p, B.grid_rst, B.max_ld, s, sto[q]));
  nl += nsto - 1;
  KSG_CUDA(launch_batch_control(B.inst.p, B.list.p, B.hdr.p, B.status.p, B.grid_inst, s));
  nl += 4;
  KSG_CUDA(cudaMemcpyAsync(B.h_status, B.status.p, sizeof(BatchStatus) * B.cap, cudaMemcpyDeviceToHost, s));
  *launches = nl;
  return 0;
}

static PetscErrorCode engine_build_graph(BatchEngine &B) {
  KSG_CUDA(batch_prepare_restart(B.max_ld));
  KSG_CUDA(batch_prepare_ds_hep(B.max_ld));
  cudaGraph_t g = nullptr;
  KSG_CUDA(cudaStreamBeginCapture(B.s, cudaStreamCaptureModeThreadLocal));
  long long nl = 0;
  PetscErrorCode ierr = engine_enqueue_cycle(B, &nl);
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

// Work lists of the live instances (between cycles: the stream is idle).  A list buffer that has to grow is
// reallocated, and the graph, which holds its address, is captured again.
static PetscErrorCode engine_upload_maps(BatchEngine &B) {
  std::vector<BatchVB> ms, md, mu, mr;
  for (int i : B.live) {
    const BatchInst &p = B.hi[i];
    const int ns = std::max(1, std::min(spmv_blocks_for(p.n, p.lanes), (p.n + 8 * SPMV_VB_ROWS - 1) / (8 * SPMV_VB_ROWS)));
    const int nd = batch_gs_vbs(p.n, gs_dot_blocks(p.n)), nu = batch_gs_vbs(p.n, gs_update_blocks(p.n));
    const int nr = std::max(1, std::min(restart_blocks_for(p.n), (p.n + 1023) / 1024));
    for (int b = 0; b < ns; ++b) ms.push_back({i, b, ns, 0});
    for (int b = 0; b < nd; ++b) md.push_back({i, b, nd, 0});
    for (int b = 0; b < nu; ++b) mu.push_back({i, b, nu, 0});
    for (int b = 0; b < nr; ++b) mr.push_back({i, b, nr, 0});
  }
  bool regrown = false;
  auto up = [&](DBuf<BatchVB> &d, const std::vector<BatchVB> &h) -> cudaError_t {
    if (h.size() > d.count || !d.p) {
      cudaError_t e = d.alloc(std::max<size_t>(h.size() + h.size() / 2 + 64, 1024));
      if (e != cudaSuccess) return e;
      regrown = true;
    }
    return h.empty() ? cudaSuccess
                     : cudaMemcpyAsync(d.p, h.data(), h.size() * sizeof(BatchVB), cudaMemcpyHostToDevice, B.s);
  };
  KSG_CUDA(cudaStreamSynchronize(B.s));
  KSG_CUDA(up(B.map_spmv, ms));
  KSG_CUDA(up(B.map_dot, md));
  KSG_CUDA(up(B.map_upd, mu));
  KSG_CUDA(up(B.map_rst, mr));
  if (!B.live.empty())
    KSG_CUDA(cudaMemcpyAsync(B.list.p, B.live.data(), B.live.size() * sizeof(int), cudaMemcpyHostToDevice, B.s));
  BatchHdr h = {};
  h.n_spmv = (int)ms.size();
  h.n_dot = (int)md.size();
  h.n_upd = (int)mu.size();
  h.n_rst = (int)mr.size();
  h.n_inst = (int)B.live.size();
  KSG_CUDA(cudaMemcpyAsync(B.hdr.p, &h, sizeof(h), cudaMemcpyHostToDevice, B.s));
  KSG_CUDA(cudaStreamSynchronize(B.s));  // h is on the stack
  if (regrown || !B.exec) KSG_TRY(engine_build_graph(B));
  B.maps_dirty = false;
  return 0;
}

// Take a set-up EPS into a free slot: start vector into column 0, instance record to the device, all on the EPS's
// own stream (the engine's stream may be running a cycle).  The instance joins the live set at ksg_engine_activate.
PetscErrorCode ksg_engine_admit(BatchEngine &B, EPS e, int *slot, double tol) {
  KSG_CHECK(!B.free_slots.empty(), PETSC_ERR_GPU_RESOURCE, "batched engine: all %d slots are in use", B.cap);
  KSG_CHECK(e->storage != STORE_F32 || B.has_f32, PETSC_ERR_PLIB, "batched engine built without the FP32 kernels");
  const int i = B.free_slots.back();
  B.free_slots.pop_back();
  B.eps[i] = e;
  B.hi[i] = make_inst(e);
  if (tol > 0.0) B.hi[i].tol = tol;
  e->solved = 0;
  e->stats = EPSGB300Stats{};
  cudaStream_t s = e->stream;
  // the start vector in FP64 into column 1, converted to pairs in column 0 (column 1 is rewritten by the first SpMV)
  std::vector<double> rnd;
  const double *src;
  if (!e->v0_internal.empty()) src = e->v0_internal.data();  // the precision form's refinement sweep
  else if (!e->v0.empty()) src = e->v0.data();
  else {
    rnd.resize(e->n);
    ksg_random_fill(rnd.data(), e->n, e->seed, 0);
    src = rnd.data();
  }
  double *stage = e->V.p + e->ldv;  // bytes [8 ldv, 16 ldv): clear of column 0 in either format
  KSG_CUDA(cudaMemcpyAsync(stage, src, sizeof(double) * e->n, cudaMemcpyHostToDevice, s));
  if (e->storage == STORE_F32) KSG_CUDA(launch_f64_to_f32(stage, reinterpret_cast<float *>(e->V.p), e->n, s));
  else KSG_CUDA(launch_f64_to_pair(stage, reinterpret_cast<float2 *>(e->V.p), e->n, s));
  KSG_CUDA(cudaMemcpyAsync(B.inst.p + i, &B.hi[i], sizeof(BatchInst), cudaMemcpyHostToDevice, s));
  KSG_CUDA(cudaStreamSynchronize(s));  // rnd and the host record go out of scope / may change
  *slot = i;
  return 0;
}

PetscErrorCode ksg_engine_activate(BatchEngine &B, const std::vector<int> &slots) {
  for (int i : slots) B.live.push_back(i);
  if (!slots.empty()) B.maps_dirty = true;
  return 0;
}

PetscErrorCode ksg_engine_launch(BatchEngine &B) {
  if (B.maps_dirty || !B.exec) KSG_TRY(engine_upload_maps(B));
  KSG_CUDA(cudaGraphLaunch(B.exec, B.s));
  B.cycles++;
  return 0;
}

// Wait for the cycle, then hand breakdowns to the single-problem code and retire solved or failed instances:
// their results go into their EPS (EPSSolve's epilogue) and their slots become free.
PetscErrorCode ksg_engine_finish(BatchEngine &B, std::vector<std::pair<int, int>> *retired) {
  KSG_CUDA(cudaStreamSynchronize(B.s));
  std::vector<int> still;
  std::vector<double> er, ei, es;
  for (int i : B.live) {
    EPS e = B.eps[i];
    int ph = B.h_status[i].phase;
    if (ph == BP_HOST) {
      // breakdown: a new random start vector at column nconv, as the single-problem loop does
      int bd = 0;
      KSG_TRY(ksg_eps_new_start_vector(e, B.h_status[i].nconv, &bd));
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
      ph = cur.phase;
    }
    if (ph == BP_START || ph == BP_ITER) {
      still.push_back(i);
      continue;
    }
    BatchInst fin;
    KSG_CUDA(cudaMemcpy(&fin, B.inst.p + i, sizeof(BatchInst), cudaMemcpyDeviceToHost));
    int err = 0;
    if (ph == BP_FAILED) {
      err = fin.err ? fin.err : PETSC_ERR_LIB;
    } else {
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
      KSG_CUDA(cudaStreamSynchronize(B.s));
      e->nconv = nconv;
      e->its = fin.its;
      e->reason = fin.reason;
      e->stats.krylov_steps = fin.steps;
      e->stats.restarts = fin.its;
      e->stats.kernel_launches = fin.its * B.launches_per_cycle;
      e->solved = 1;
      e->xvec_valid = 0;
    }
    retired->push_back({i, err});
    B.eps[i] = nullptr;
    B.free_slots.push_back(i);
    B.maps_dirty = true;
  }
  B.live.swap(still);
  return 0;
}

}  // namespace ksg

using namespace ksg;

extern "C" PetscErrorCode EPSGB300SolveBatch(PetscInt count, EPS *eps) {
  KSG_CHECK(count >= 0, PETSC_ERR_ARG_OUTOFRANGE, "Negative count");
  if (count == 0) return 0;
  KSG_CHECK(eps, PETSC_ERR_ARG_NULL, "Null EPS array");
  auto t0 = std::chrono::steady_clock::now();
  int device = -1, max_ncv = 1;
  bool any_f32 = false;
  for (int i = 0; i < count; ++i) {
    KSG_CHECK(eps[i], PETSC_ERR_ARG_NULL, "Null EPS at position %d", i);
    KSG_TRY(EPSSetUp(eps[i]));
    KSG_TRY(ksg_engine_check(eps[i], batch_max_columns() - 1, true));
    any_f32 = any_f32 || eps[i]->arith == ARITH_F32;
    max_ncv = std::max(max_ncv, eps[i]->ncv_e);
    if (device < 0) device = eps[i]->device;
    KSG_CHECK(eps[i]->device == device, PETSC_ERR_ARG_INCOMP, "EPSGB300SolveBatch: all EPS must use one device");
    for (int j = 0; j < i; ++j) KSG_CHECK(eps[j] != eps[i], PETSC_ERR_ARG_WRONG, "EPS %d appears twice", i);
  }
  KSG_CUDA(cudaSetDevice(device));
  KSG_CUDA(cudaDeviceSynchronize());  // EPSSetUp work on the objects' own streams
  BatchEngine B;
  KSG_TRY(ksg_engine_init(B, device, (int)count, max_ncv, any_f32));
  // the precision form runs its FP32 phase first (to max(tol, 1e-6)), then, after the FP64 recheck, either widens
  // the basis or goes through the engine again as an FP64-class refinement sweep (EPSSolve's precision driver)
  std::vector<int> slot_of(count), stage(count, 0);  // stage: 0 plain, 1 FP32 phase, 2 refinement sweep
  std::vector<long long> psteps(count, 0), pits(count, 0);
  std::vector<int> owner(count, -1);
  std::vector<int> first;
  for (int i = 0; i < count; ++i) {
    EPS e = eps[i];
    double tol = 0.0;
    if (e->arith == ARITH_F32) {
      e->storage = STORE_F32;
      stage[i] = 1;
      tol = std::max(e->tol_e, 1e-6);
    }
    KSG_TRY(ksg_engine_admit(B, e, &slot_of[i], tol));
    owner[slot_of[i]] = i;
    first.push_back(slot_of[i]);
  }
  KSG_TRY(ksg_engine_activate(B, first));
  std::vector<std::pair<int, int>> retired;
  int first_err = 0, err_at = -1;
  while (!B.live.empty()) {
    KSG_TRY(ksg_engine_launch(B));
    retired.clear();
    KSG_TRY(ksg_engine_finish(B, &retired));
    std::vector<int> again;
    for (auto &r : retired) {
      const int i = owner[r.first];
      owner[r.first] = -1;
      if (r.second) {
        if (!first_err) {
          first_err = r.second;
          err_at = i;
        }
        continue;
      }
      EPS e = eps[i];
      if (stage[i] == 1) {
        psteps[i] = e->stats.krylov_steps;
        pits[i] = e->its;
        bool pass = e->reason == 1;
        for (int k = 0; k < std::min(e->nconv, e->nev_e) && pass; ++k) {
          double err = 0.0;
          KSG_TRY(EPSComputeError(e, k, EPS_ERROR_RELATIVE, &err));
          if (!(err <= e->tol_e)) pass = false;
        }
        if (pass) {
          KSG_TRY(ksg_eps_widen_f32(e, e->nconv));
          e->storage = STORE_PAIR;
          e->stats.precision_steps = psteps[i];
          e->stats.precision_restarts = pits[i];
          stage[i] = 0;
        } else {
          std::vector<double> acc(e->n, 0.0), col(e->n);
          const int use = std::max(1, std::min(e->nconv, e->nev_e));
          for (int k = 0; k < use && k < e->nconv; ++k) {
            KSG_TRY(ksg_get_column(col.data(), ksg_col(e->V.p, e->ldv, e->perm[k], STORE_F32), e->n, STORE_F32,
                                   e->stream));
            for (int r2 = 0; r2 < e->n; ++r2) acc[r2] += col[r2];
          }
          e->v0_internal.swap(acc);
          e->storage = STORE_PAIR;
          stage[i] = 2;
          int sl = -1;
          KSG_TRY(ksg_engine_admit(B, e, &sl, 0.0));
          owner[sl] = i;
          again.push_back(sl);
        }
      } else if (stage[i] == 2) {
        e->v0_internal.clear();
        e->stats.precision_steps = psteps[i];
        e->stats.precision_restarts = pits[i];
        e->stats.krylov_steps += psteps[i];
        e->its += (int)pits[i];
        stage[i] = 0;
      }
    }
    if (!again.empty()) KSG_TRY(ksg_engine_activate(B, again));
  }
  const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  for (int i = 0; i < count; ++i) {
    eps[i]->stats.solve_seconds = secs;
    eps[i]->stats.kernel_launches = B.cycles * B.launches_per_cycle;
  }
  KSG_CHECK(!first_err, first_err, "EPSGB300SolveBatch: problem %d failed (%s)", err_at,
            first_err == 77 ? "initial vector is zero or the Krylov segment is empty"
                            : "the projected eigenproblem solver did not converge");
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
