// api_noalloc.cu -- BVGB300DotVecNoAlloc: y = V^T x on device data, with no device memory allocated by the call.
//
// Some callers cannot allocate device memory while they run: an application that reserves all GPU memory up front
// for its own pool allocator (a cudaMalloc outside that pool can fail or fragment it), or a time-critical loop that
// cannot afford the implicit device synchronisation of cudaMalloc/cudaFree.  For them this entry point runs the dot
// half of the Gram-Schmidt pair (the kernel behind BVDotVec) with its scratch -- the per-block partial sums, the
// last-block ticket counter and the staging of the results -- in the fixed array below, which every GPU that loads
// this library holds until the process exits.
#include <stdint.h>

#include <mutex>

#include "internal.h"

using namespace ksg;

namespace {
constexpr int NA_MAX_COLS = 256;     // largest k accepted
constexpr int NA_MAX_BLOCKS = 160;   // the dot kernel's grid is capped here (one block per SM on GB300's 152 SMs)
constexpr int NA_PART_STRIDE = NA_MAX_COLS + 8;  // partial sums per block (k values + u.u), 8-byte units
constexpr size_t NA_STATE_BYTES = 256;
constexpr size_t NA_COEF_BYTES = (size_t)(2 * NA_MAX_COLS + 8) * 8;
constexpr size_t NA_PART_BYTES = (size_t)NA_MAX_BLOCKS * NA_PART_STRIDE * 8;
constexpr size_t NA_SCRATCH_BYTES = NA_STATE_BYTES + NA_COEF_BYTES + NA_PART_BYTES;  // 344,448 bytes
static_assert(sizeof(KrylovState) <= NA_STATE_BYTES, "state does not fit its slot");
constexpr int NA_MAX_DEVICES = 64;

std::mutex g_na_mutex;
unsigned char *g_na_addr[NA_MAX_DEVICES] = {nullptr};
}  // namespace

// The scratch itself.  In host code this name is only a host-side stand-in for the symbol, never a device address:
// the device address is obtained once per device with cudaGetSymbolAddress below.
static __device__ __align__(256) unsigned char g_noalloc_scratch[NA_SCRATCH_BYTES];

// Device address of the scratch on the current device, looked up on the first call made on that device.
static PetscErrorCode na_scratch(unsigned char **out) {
  int dev = 0;
  KSG_CUDA(cudaGetDevice(&dev));
  KSG_CHECK(dev >= 0 && dev < NA_MAX_DEVICES, PETSC_ERR_SUP, "Device ordinal %d above %d", dev, NA_MAX_DEVICES - 1);
  std::lock_guard<std::mutex> lock(g_na_mutex);
  if (!g_na_addr[dev]) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p)
      return ksg_set_error(PETSC_ERR_GPU, "cudaGetSymbolAddress of the no-allocation scratch failed on device %d: %s",
                           dev, cudaGetErrorString(e));
    g_na_addr[dev] = static_cast<unsigned char *>(p);
  }
  *out = g_na_addr[dev];
  return 0;
}

extern "C" PetscErrorCode BVGB300DotVecNoAlloc(const double *V, PetscInt ldv, PetscInt n, PetscInt k, const double *x,
                                               double *y, void *stream) {
  KSG_CHECK(x && y && (V || k == 0), PETSC_ERR_ARG_NULL, "Null device pointer");
  KSG_CHECK(n > 0, PETSC_ERR_ARG_OUTOFRANGE, "n must be positive");
  KSG_CHECK(k >= 0 && k <= NA_MAX_COLS, PETSC_ERR_ARG_OUTOFRANGE,
            "k = %d columns exceeds the fixed scratch of this entry point (at most %d)", k, NA_MAX_COLS);
  KSG_CHECK(ldv >= n && (ldv % 2) == 0, PETSC_ERR_ARG_WRONG, "ldv must be even and at least n");
  KSG_CHECK(((uintptr_t)V % 16) == 0, PETSC_ERR_ARG_WRONG, "V must be 16-byte aligned");
  if (k == 0) return 0;
  unsigned char *base = nullptr;
  KSG_TRY(na_scratch(&base));
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  KrylovState *st = reinterpret_cast<KrylovState *>(base);
  double *coef = reinterpret_cast<double *>(base + NA_STATE_BYTES);
  float2 *part = reinterpret_cast<float2 *>(base + NA_STATE_BYTES + NA_COEF_BYTES);
  // the array keeps the previous call's contents: the ticket counter must start at zero, the scale at one
  KSG_CUDA(cudaMemsetAsync(st, 0, NA_STATE_BYTES, s));
  KSG_CUDA(launch_segment_begin(st, 0, 0, s));
  StepArgs a = {};
  a.V = V;
  a.ldv = ldv;
  a.n = n;
  a.J = k;
  a.j = k;
  a.hermitian = 1;
  a.U = const_cast<double *>(x);  // read only in this mode
  a.W = nullptr;
  a.eta = 0.7071;
  a.coef = coef;
  a.part = part;
  a.pstride = NA_PART_STRIDE;
  a.st = st;
  // a device with more SMs than the scratch has block slots runs the kernel on NA_MAX_BLOCKS blocks, which loop
  // over the row tiles: any n works on any device
  KSG_CUDA(launch_gs_dot(a, 1, GS_DOTS, ARITH_PAIR, s, STORE_F64, NA_MAX_BLOCKS));
  KSG_CUDA(cudaMemcpyAsync(y, coef, sizeof(double) * k, cudaMemcpyDeviceToDevice, s));
  return 0;
}
