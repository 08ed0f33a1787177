// k_batch.cu -- the batched Krylov-Schur engine: every live instance of a batch advances one Krylov step per launch.
//
// Each kernel runs a persistent grid over a list of virtual blocks (instance, b, nb): virtual block b of nb is the
// share instance `inst` would get from block b of an nb-block launch of the single-problem kernel, and it runs the
// same device body (krylov_body.cuh).  An instance's arithmetic therefore depends only on its own size -- the
// result of a problem solved inside any mix equals its result solved alone in a batch of one.  Instances that
// are not in the phase a launch serves skip their virtual blocks at once, so one captured sequence of launches (a
// restart cycle) serves every cycle of every instance:
//
//   k_batch_zero + start pass (GS_ORTHO on column 0) + k_batch_start  -> newly admitted instances enter ITER
//   slot s = 0 .. S:  k_batch_spmv(s), k_batch_dot(s), k_batch_update(s)   (instance steps if k0 <= s < nv,
//                                                                            final reorthogonalisation if s == nv)
//   projected problems (k_ds_hep.cu / k_ds_nhep.cu batched kernels), k_batch_restart, k_batch_control
//
// k_batch_control is the device copy of the host loop of EPSSolve_KrylovSchur_Default (krylovschur.c:227-337):
// it reads the control record the projected solver wrote and sets up the next segment.
#include "batch_types.h"
#include "common.cuh"
#include "kernels.h"
#include "krylov_body.cuh"
#include "ks_types.h"

namespace ksg {

KS_DEVICE void batch_segment_begin(KrylovState *st, int k0, int m) {
  st->sigma = 1.0;
  st->beta_prev = 0.0;
  st->invnu = 1.0;
  st->tau_sigma = 0.0;
  st->beta_out = 0.0;
  st->onorm = 0.0;
  st->stop = 0;
  st->m = m;
  st->breakdown = 0;
  st->k0 = k0;
}

// The Gram-Schmidt work of instance p in slot `slot`: mode and NX, or false if it has none.
KS_DEVICE bool batch_slot(const BatchInst &p, int slot, int &mode, int &nx, int &j) {
  if (slot < 0) {  // start pass: normalise column 0
    if (p.phase != BP_START) return false;
    mode = GS_ORTHO;
    nx = 1;
    j = 0;
    return true;
  }
  if (p.phase != BP_ITER) return false;
  if (slot >= p.k0 && slot < p.nv) {
    mode = GS_STEP;
    nx = 2;
    j = slot;
    return true;
  }
  if (slot == p.nv) {
    mode = GS_FINAL;
    nx = 1;
    j = slot;
    return true;
  }
  return false;
}

// basis column j of instance p (8 bytes per entry, 4 for the precision form's FP32 phase)
template <int STO = -1>
KS_DEVICE void *batch_col(const BatchInst &p, int j) {
  const size_t es = (STO == STORE_F32 || (STO < 0 && p.storage == STORE_F32)) ? 4 : 8;
  return reinterpret_cast<char *>(p.V) + (size_t)j * (size_t)p.ldv * es;
}

template <int STO>
KS_DEVICE StepArgs batch_step_args(const BatchInst &p, int j, int nx) {
  StepArgs a = {};  // no constraint columns (nc = 0) in the batched engine
  a.V = p.V;
  a.ldv = p.ldv;
  a.n = p.n;
  a.J = j;
  a.j = j;
  a.hermitian = p.hermitian;
  a.U = batch_col<STO>(p, j);
  a.W = (nx == 2) ? batch_col<STO>(p, j + 1) : nullptr;
  a.d = p.d;
  a.e = p.e;
  a.H = p.H;
  a.ldh = p.ld;
  a.eta = 0.7071;
  a.coef = p.coef;
  a.part = p.part;
  a.pstride = p.pstride;
  a.st = p.st;
  return a;
}

// zero d, e and H of newly admitted instances, reset their Krylov state for the start pass
__global__ void k_batch_zero(BatchInst *I, const int *list, const BatchHdr *h) {
  for (int v = blockIdx.x; v < h->n_inst; v += gridDim.x) {
    BatchInst &p = I[list[v]];
    if (p.phase != BP_START) continue;
    const int ld = p.ld;
    for (int i = threadIdx.x; i < ld + 1; i += blockDim.x) {
      p.d[i] = 0.0;
      p.e[i] = 0.0;
    }
    for (int i = threadIdx.x; i < (ld + 1) * (ld + 1); i += blockDim.x) p.H[i] = 0.0;
    if (threadIdx.x == 0) batch_segment_begin(p.st, 0, 0);
  }
}

// after the start pass: ITER, or FAILED if the start vector is zero (EPSSolve's "Initial vector is zero")
__global__ void k_batch_start(BatchInst *I, const int *list, const BatchHdr *h) {
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < h->n_inst; v += gridDim.x * blockDim.x) {
    BatchInst &p = I[list[v]];
    if (p.phase != BP_START) continue;
    if (p.st->breakdown) {
      p.phase = BP_FAILED;
      p.err = 77;  // PETSC_ERR_PLIB, as the single-problem path reports a zero initial vector
      continue;
    }
    p.phase = BP_ITER;
    p.nconv = 0;
    p.l = 0;
    p.its = 1;
    p.reason = 0;
    p.steps = 0;
    p.k0 = 0;
    p.nv = min(p.mpd, p.ncv);
    batch_segment_begin(p.st, 0, p.nv);
  }
}

template <int LANES>
KS_DEVICE void batch_spmv_vb(const BatchInst &p, const BatchVB &m, int slot) {
  const long long w0 = (long long)m.b * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const long long nw = (long long)m.nb * (blockDim.x >> 5);
  if (p.storage == STORE_F32)
    spmv_f32_rows<LANES>(p.rp, p.ci, p.va32, static_cast<const float *>(batch_col(p, slot)),
                         static_cast<float *>(batch_col(p, slot + 1)), p.n, p.st, p.opscale, w0, nw);
  else
    spmv_pair_rows<LANES>(p.rp, p.ci, p.va2, static_cast<const float2 *>(batch_col(p, slot)),
                          static_cast<float2 *>(batch_col(p, slot + 1)), p.n, p.st, p.opscale, w0, nw);
}

// each batched kernel serves the instances of one storage format (STO); the others skip their virtual blocks
template <int STO>
__global__ void __launch_bounds__(256) k_batch_spmv(const BatchInst *I, const BatchVB *map, const BatchHdr *h,
                                                    int slot) {
  const int nmap = h->n_spmv;
  for (int v = blockIdx.x; v < nmap; v += gridDim.x) {
    const BatchVB m = map[v];
    const BatchInst &p = I[m.inst];
    if (p.storage != STO || p.phase != BP_ITER || slot < p.k0 || slot >= p.nv) continue;
    switch (p.lanes) {
      case 1: batch_spmv_vb<1>(p, m, slot); break;
      case 8: batch_spmv_vb<8>(p, m, slot); break;
      default: batch_spmv_vb<32>(p, m, slot); break;
    }
  }
}

// Gram-Schmidt half A; CPW = 5 covers engines of up to 80 columns, CPW = 9 up to 144 (the per-column arithmetic
// does not depend on CPW, so both match the single-problem kernel's rounding)
constexpr int BATCH_CPW = 5;
constexpr int BATCH_CPW_WIDE = 9;
constexpr int BATCH_MAXJ = A_WARPS * BATCH_CPW_WIDE;

template <int STO, class S, int CPW>
__global__ void __launch_bounds__(A_THREADS, 1) k_batch_dot(const BatchInst *I, const BatchVB *map,
                                                            const BatchHdr *h, int slot) {
  const int nmap = h->n_dot;
  for (int v = blockIdx.x; v < nmap; v += gridDim.x) {
    const BatchVB m = map[v];
    const BatchInst &p = I[m.inst];
    int mode, nx, j;
    if (p.storage != STO || !batch_slot(p, slot, mode, nx, j)) continue;
    __syncthreads();  // shared staging of the previous virtual block is free
    const StepArgs a = batch_step_args<STO>(p, j, nx);
    if (nx == 2) gs_dot_body<2, CPW, PairAr, S>(a, mode, m.b, m.nb);
    else gs_dot_body<1, CPW, PairAr, S>(a, mode, m.b, m.nb);
  }
}

template <int STO, class S>
__global__ void __launch_bounds__(B_THREADS, 2) k_batch_update(const BatchInst *I, const BatchVB *map,
                                                            const BatchHdr *h, int slot) {
  const int nmap = h->n_upd;
  for (int v = blockIdx.x; v < nmap; v += gridDim.x) {
    const BatchVB m = map[v];
    const BatchInst &p = I[m.inst];
    int mode, nx, j;
    if (p.storage != STO || !batch_slot(p, slot, mode, nx, j)) continue;
    __syncthreads();
    const StepArgs a = batch_step_args<STO>(p, j, nx);
    if (nx == 2) gs_update_body<2, PairAr, S>(a, mode, m.b, m.nb);
    else gs_update_body<1, PairAr, S>(a, mode, m.b, m.nb);
  }
}

// Thick restart V(:, nconv : k+l) = V(:, nconv : nv) Q(nconv : nv, nconv : k+l), then the residual column moves to
// column k+l (krylovschur.c:300-329), for every instance whose projected problem was solved this cycle.
template <int STO, int CQ>
__global__ void __launch_bounds__(R_THREADS, 2) k_batch_restart(const BatchInst *I, const BatchVB *map,
                                                                const BatchHdr *h) {
  constexpr int TR = restart_tile_rows<CQ>();
  const int nmap = h->n_rst;
  for (int v = blockIdx.x; v < nmap; v += gridDim.x) {
    const BatchVB m = map[v];
    const BatchInst &p = I[m.inst];
    if (p.storage != STO || p.phase != BP_ITER) continue;
    const KSControl c = *p.ctl;
    if (c.ds_error) continue;
    const int k = c.nconv, l = c.l, nv = c.nv, nconv = p.nconv;
    const int K = nv - nconv, N = k + l - nconv;
    __syncthreads();
    if (K > 0 && N > 0) {
      if (STO == STORE_F32)
        restart_body<PairAr, StF32, CQ>(static_cast<float *>(batch_col(p, 0)), p.ldv, p.n, nconv, K, nconv, N, p.Q,
                                        p.ld, m.b, m.nb);
      else
        restart_body<PairAr, StPair, CQ>(p.V, p.ldv, p.n, nconv, K, nconv, N, p.Q, p.ld, m.b, m.nb);
    }
    if (c.reason == 0 && !(c.breakdown || k == nv)) {
      // this virtual block's rows only (the restart's row tiles): the restart above already consumed column k+l
      // for them
      const int ntiles = (p.n + TR - 1) / TR;
      const bool f32 = STO == STORE_F32;
      for (int t = m.b; t < ntiles; t += m.nb) {
        const int rend = min(p.n, (t + 1) * TR);
        for (int r = t * TR + threadIdx.x; r < rend; r += R_THREADS) {
          if (f32) static_cast<float *>(batch_col(p, k + l))[r] = static_cast<const float *>(batch_col(p, nv))[r];
          else static_cast<float2 *>(batch_col(p, k + l))[r] = static_cast<const float2 *>(batch_col(p, nv))[r];
        }
      }
    }
  }
}

// One thread per instance: the restart-loop bookkeeping of EPSSolve_KrylovSchur_Default after the restart.
__global__ void k_batch_control(BatchInst *I, const int *list, const BatchHdr *h, BatchStatus *status) {
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < h->n_inst; v += gridDim.x * blockDim.x) {
    const int i = list[v];
    BatchInst &p = I[i];
    if (p.phase == BP_ITER) {
      const KSControl c = *p.ctl;
      p.steps += (c.nv > p.k0) ? c.nv - p.k0 : 0;
      if (c.ds_error) {
        p.phase = BP_FAILED;
        p.err = 76;  // PETSC_ERR_LIB: the projected eigenproblem solver did not converge
      } else {
        const int k = c.nconv;
        p.nconv = k;
        p.l = c.l;
        p.reason = c.reason;
        if (c.reason != 0) {
          p.phase = BP_DONE;
        } else {
          p.its += 1;
          p.k0 = k + c.l;
          p.nv = min(k + p.mpd, p.ncv);
          if (c.breakdown || k == c.nv) p.phase = BP_HOST;  // new start vector at column k (host)
          else if (p.nv <= p.k0) {
            p.phase = BP_FAILED;
            p.err = 77;
          } else batch_segment_begin(p.st, p.k0, p.nv);
        }
      }
    }
    BatchStatus s;
    s.phase = p.phase;
    s.nconv = p.nconv;
    s.its = p.its;
    s.reason = p.reason;
    status[i] = s;
  }
}

// ---------------------------------------------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------------------------------------------
int batch_max_columns() { return BATCH_MAXJ; }

cudaError_t launch_batch_begin(BatchInst *I, const int *list, const BatchHdr *h, int grid_inst, cudaStream_t s) {
  k_batch_zero<<<grid_inst, 256, 0, s>>>(I, list, h);
  return cudaGetLastError();
}

cudaError_t launch_batch_start(BatchInst *I, const int *list, const BatchHdr *h, int grid_inst, cudaStream_t s) {
  k_batch_start<<<(grid_inst + 127) / 128, 128, 0, s>>>(I, list, h);
  return cudaGetLastError();
}

cudaError_t launch_batch_spmv(const BatchInst *I, const BatchVB *map, const BatchHdr *h, int slot, int grid,
                              cudaStream_t s, int storage) {
  if (storage == STORE_F32) k_batch_spmv<STORE_F32><<<grid, 256, 0, s>>>(I, map, h, slot);
  else k_batch_spmv<STORE_PAIR><<<grid, 256, 0, s>>>(I, map, h, slot);
  return cudaGetLastError();
}

cudaError_t launch_batch_dot(const BatchInst *I, const BatchVB *map, const BatchHdr *h, int slot, int grid,
                             cudaStream_t s, int storage, int max_ld) {
  if (max_ld > BATCH_MAXJ) return cudaErrorInvalidValue;
  if (max_ld <= A_WARPS * BATCH_CPW) {
    if (storage == STORE_F32) k_batch_dot<STORE_F32, StF32, BATCH_CPW><<<grid, A_THREADS, 0, s>>>(I, map, h, slot);
    else k_batch_dot<STORE_PAIR, StPair, BATCH_CPW><<<grid, A_THREADS, 0, s>>>(I, map, h, slot);
  } else {
    if (storage == STORE_F32)
      k_batch_dot<STORE_F32, StF32, BATCH_CPW_WIDE><<<grid, A_THREADS, 0, s>>>(I, map, h, slot);
    else k_batch_dot<STORE_PAIR, StPair, BATCH_CPW_WIDE><<<grid, A_THREADS, 0, s>>>(I, map, h, slot);
  }
  return cudaGetLastError();
}

cudaError_t launch_batch_update(const BatchInst *I, const BatchVB *map, const BatchHdr *h, int slot, int grid,
                                int max_ld, cudaStream_t s, int storage) {
  const size_t shm = (size_t)2 * max_ld * sizeof(f2x);
  if (storage == STORE_F32) k_batch_update<STORE_F32, StF32><<<grid, B_THREADS, shm, s>>>(I, map, h, slot);
  else k_batch_update<STORE_PAIR, StPair><<<grid, B_THREADS, shm, s>>>(I, map, h, slot);
  return cudaGetLastError();
}

// the restart variant for the engine's widest instance: N <= max_ld - 1 columns
template <int CQ>
static size_t batch_restart_smem(int max_ld) { return restart_smem_bytes(max_ld, max_ld, restart_tile_rows<CQ>()); }

template <int CQ>
static cudaError_t batch_restart_attrs(int max_ld) {
  const int shm = (int)batch_restart_smem<CQ>(max_ld);
  cudaError_t e = cudaFuncSetAttribute(k_batch_restart<STORE_PAIR, CQ>, cudaFuncAttributeMaxDynamicSharedMemorySize, shm);
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(k_batch_restart<STORE_F32, CQ>, cudaFuncAttributeMaxDynamicSharedMemorySize, shm);
}

template <int CQ>
static cudaError_t batch_restart_go(const BatchInst *I, const BatchVB *map, const BatchHdr *h, int grid, int max_ld,
                                    cudaStream_t s, int storage) {
  const size_t shm = batch_restart_smem<CQ>(max_ld);
  if (storage == STORE_F32) k_batch_restart<STORE_F32, CQ><<<grid, R_THREADS, shm, s>>>(I, map, h);
  else k_batch_restart<STORE_PAIR, CQ><<<grid, R_THREADS, shm, s>>>(I, map, h);
  return cudaGetLastError();
}

// kernel attributes, set before a cycle is captured
cudaError_t batch_prepare_restart(int max_ld) {
  const int nmax = max_ld - 1;
  if (nmax <= 16) return batch_restart_attrs<1>(max_ld);
  if (nmax <= 32) return batch_restart_attrs<2>(max_ld);
  if (nmax <= 64) return batch_restart_attrs<4>(max_ld);
  return batch_restart_attrs<9>(max_ld);
}

cudaError_t launch_batch_restart(const BatchInst *I, const BatchVB *map, const BatchHdr *h, int grid, int max_ld,
                                 cudaStream_t s, int storage) {
  const int nmax = max_ld - 1;
  if (nmax <= 16) return batch_restart_go<1>(I, map, h, grid, max_ld, s, storage);
  if (nmax <= 32) return batch_restart_go<2>(I, map, h, grid, max_ld, s, storage);
  if (nmax <= 64) return batch_restart_go<4>(I, map, h, grid, max_ld, s, storage);
  return batch_restart_go<9>(I, map, h, grid, max_ld, s, storage);
}

cudaError_t launch_batch_control(BatchInst *I, const int *list, const BatchHdr *h, BatchStatus *status,
                                 int grid_inst, cudaStream_t s) {
  k_batch_control<<<(grid_inst + 127) / 128, 128, 0, s>>>(I, list, h, status);
  return cudaGetLastError();
}

}  // namespace ksg
