// batch_engine.h -- host side of the batched Krylov-Schur engine, shared by EPSGB300SolveBatch and the server.
//
// The engine owns a fixed number of instance slots.  An EPS that EPSSetUp prepared is admitted into a free slot
// (its start vector and instance record go to the device on the EPS's own stream), activated into the live set
// between cycles, advanced by restart cycles (one CUDA graph launch each), and retired when its restart loop ends:
// its results are written into the EPS exactly as EPSSolve would, and the slot is free again.
#pragma once

#include <utility>
#include <vector>

#include "batch_types.h"
#include "internal.h"

namespace ksg {

struct BatchEngine {
  int device = 0;
  int cap = 0;     // instance slots
  int slots = 0;   // Gram-Schmidt slots per cycle: ncv limit + 1 (steps 0..ncv-1, final pass at nv <= ncv)
  int max_ld = 0;  // ncv limit + 1
  int grid_spmv = 0, grid_dot = 0, grid_upd = 0, grid_rst = 0, grid_ds = 0, grid_inst = 0;
  cudaStream_t s = nullptr;
  DBuf<BatchInst> inst;
  DBuf<BatchVB> map_spmv, map_dot, map_upd, map_rst;
  DBuf<int> list;
  DBuf<BatchHdr> hdr;
  DBuf<BatchStatus> status;
  BatchStatus *h_status = nullptr;  // pinned, written by the last node of each cycle
  cudaGraphExec_t exec = nullptr;
  long long launches_per_cycle = 0;
  long long cycles = 0;
  bool maps_dirty = true;
  bool has_f32 = false;  // the cycle graph includes the FP32-storage kernels
  std::vector<BatchInst> hi;  // host copy of each slot's problem fields
  std::vector<EPS> eps;       // slot -> EPS (nullptr when free)
  std::vector<int> live;      // slots in the live set
  std::vector<int> free_slots;
  ~BatchEngine();
};

PetscErrorCode ksg_engine_check(EPS e, int max_ncv, bool allow_f32);
PetscErrorCode ksg_engine_init(BatchEngine &B, int device, int cap, int max_ncv, bool with_f32 = false);
// tol > 0 overrides the EPS tolerance (the precision form's FP32 phase)
PetscErrorCode ksg_engine_admit(BatchEngine &B, EPS e, int *slot, double tol = 0.0);
PetscErrorCode ksg_engine_activate(BatchEngine &B, const std::vector<int> &slots);
PetscErrorCode ksg_engine_launch(BatchEngine &B);
// retired: (slot, PETSc error code or 0) of every instance whose restart loop ended in this cycle
PetscErrorCode ksg_engine_finish(BatchEngine &B, std::vector<std::pair<int, int>> *retired);

}  // namespace ksg
