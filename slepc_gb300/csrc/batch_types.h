// batch_types.h -- device records of the batched Krylov-Schur engine: many independent eigenproblems advance
// together, one Krylov step of every live instance per launch, one restart cycle per CUDA graph launch.
#pragma once

#include <cuda_runtime.h>

#include "kernels.h"
#include "ks_types.h"

namespace ksg {

// Instance life cycle.  START: the start vector still has to be normalised; ITER: inside the restart loop;
// HOST: the factorisation broke down and the host draws a new start vector; DONE / FAILED: retired.
enum BatchPhase : int { BP_START = 0, BP_ITER = 1, BP_HOST = 2, BP_DONE = 3, BP_FAILED = 4 };

// One eigenproblem of a batch.  The problem fields and buffers are those of its EPS (EPSSetUp allocated them);
// the cycle fields are advanced on the device by k_batch_control.
struct BatchInst {
  int n, hermitian, which, nev, ncv, mpd, max_it, lock, lanes, ld;
  double tol, keep, opscale;
  const int *rp, *ci;
  const float2 *va2;
  const float *va32;  // the precision form's FP32 values (storage STORE_F32)
  float2 *V;          // the basis; STORE_F32 instances read it as float with the same leading dimension
  long long ldv;
  int storage;        // STORE_PAIR or STORE_F32
  double *d, *e, *H, *Q, *eigr, *eigi, *errest, *coef, *work;
  float2 *part;
  int pstride;
  KrylovState *st;
  KSControl *ctl;
  // cycle state
  int phase;
  int k0, nv;         // the Krylov segment of the current cycle: steps k0 .. nv-1
  int nconv, l;       // converged (locked) and kept columns before the current cycle's restart
  int its, reason, err;
  long long steps;    // Krylov steps taken (operator applications inside factorisations)
};

// A virtual block: block b of the nb blocks that instance `inst` uses in one kernel.
struct BatchVB {
  int inst, b, nb, pad;
};

// Sizes of the work lists, read by every batched kernel (kept on the device so a captured graph stays valid when
// the live set changes).
struct BatchHdr {
  int n_spmv, n_dot, n_upd, n_rst, n_inst, pad[3];
};

// Per-instance summary the host reads once per cycle.
struct BatchStatus {
  int phase, nconv, its, reason;
};

// launchers (k_batch.cu, k_ds_hep.cu, k_ds_nhep.cu); `grid` is the persistent grid, the work lists are on the device
int batch_max_columns();
cudaError_t launch_batch_begin(BatchInst *I, const int *list, const BatchHdr *h, int grid_inst, cudaStream_t s);
cudaError_t launch_batch_start(BatchInst *I, const int *list, const BatchHdr *h, int grid_inst, cudaStream_t s);
// the Krylov-step and restart launchers serve the instances of one storage format (STORE_PAIR or STORE_F32)
cudaError_t launch_batch_spmv(const BatchInst *I, const BatchVB *map, const BatchHdr *h, int slot, int grid,
                              cudaStream_t s, int storage);
// the engine's widest basis max_ld selects the column tiling (up to 80 or up to 144 columns)
cudaError_t launch_batch_dot(const BatchInst *I, const BatchVB *map, const BatchHdr *h, int slot, int grid,
                             cudaStream_t s, int storage, int max_ld);
cudaError_t launch_batch_update(const BatchInst *I, const BatchVB *map, const BatchHdr *h, int slot, int grid,
                                int max_ld, cudaStream_t s, int storage);
cudaError_t launch_batch_restart(const BatchInst *I, const BatchVB *map, const BatchHdr *h, int grid, int max_ld,
                                 cudaStream_t s, int storage);
cudaError_t launch_batch_control(BatchInst *I, const int *list, const BatchHdr *h, BatchStatus *status,
                                 int grid_inst, cudaStream_t s);
cudaError_t launch_batch_ds_hep(const BatchInst *I, const int *list, const BatchHdr *h, int grid, int max_ld,
                                cudaStream_t s);
cudaError_t launch_batch_ds_nhep(const BatchInst *I, const int *list, const BatchHdr *h, int grid, int max_ld,
                                 cudaStream_t s);
cudaError_t batch_prepare_restart(int max_ld);
cudaError_t batch_prepare_ds_hep(int max_ld);
int spmv_blocks_for(int n, int lanes);
int restart_blocks_for(int n);

#ifdef __CUDACC__
// DSArgs of instance p for the full projected-problem step of a restart (the EPSSolve loop's DS call)
__device__ __forceinline__ DSArgs batch_ds_args(const BatchInst &p) {
  DSArgs a = {};
  a.ld = p.ld;
  a.n = p.nv;
  a.flags = DS_DO_ALL;
  a.l = p.nconv;
  a.k = p.k0;
  a.raw = p.l > 0;
  a.d = p.d;
  a.e = p.e;
  a.H = p.H;
  a.Q = p.Q;
  a.eigr = p.eigr;
  a.eigi = p.eigi;
  a.errest = p.errest;
  a.work = p.work;
  a.which = p.which;
  a.tol = p.tol;
  a.nev = p.nev;
  a.its = p.its;
  a.max_it = p.max_it;
  a.keep = p.keep;
  a.lock = p.lock;
  a.st = p.st;
  a.ctl = p.ctl;
  return a;
}
#endif

}  // namespace ksg
