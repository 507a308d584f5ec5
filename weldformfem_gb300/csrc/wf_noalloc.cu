// Nodal volumes without any device allocation.
//
// Some callers cannot call cudaMalloc: code that runs inside another
// framework's memory pool (where a raw allocation would bypass its
// accounting), real-time or long-running loops that must not risk the
// implicit device synchronisation cudaMalloc/cudaFree can cause, and hosts
// that run with a fixed device-memory budget reserved up front. For them this
// file provides wf_nodal_volumes_noalloc: the element-volume pass followed by
// the per-node volume sum (the geometry and nodal phases of the FP64 step),
// with the caller passing every input and the output buffer, and the
// element-volume scratch held in a file-scope static device array instead of
// an allocation.
//
// The scratch array below is part of the library image: every GPU that loads
// the library holds it (WF_NOALLOC_MAX_ELEMS doubles = 8 MiB) until the
// process exits. All calls share it and it keeps the last call's contents;
// every element slot a call reads is written by that same call first, so
// nothing needs clearing. Calls whose kernels overlap on the GPU (different
// streams, or host threads without ordering) race on the array.
#include <cuda.h>
#include <cuda_runtime.h>

#include <mutex>

#include "wf.h"

namespace {

constexpr int kThreads = 256;

// Element volumes of the most recent call (file-scope: no allocation).
static __device__ __align__(256) double g_vol_scratch[WF_NOALLOC_MAX_ELEMS];

// Device address of g_vol_scratch per device, with the id of the CUDA context
// it was resolved in: resolved once per device, and again only when the
// device's context has changed (after a cudaDeviceReset the old address
// belongs to a destroyed context).
constexpr int kMaxDevices = 64;
struct ScratchAddr {
  double *ptr = nullptr;
  unsigned long long ctx_id = 0;
};
ScratchAddr g_scratch_addr[kMaxDevices];
std::mutex g_scratch_mu;

// cuCtxGetCurrent / cuCtxGetId through the runtime's driver entry points (no
// link against the driver library).
using CtxGetCurrentFn = CUresult(CUDAAPI *)(CUcontext *);
using CtxGetIdFn = CUresult(CUDAAPI *)(CUcontext, unsigned long long *);

// Id of the calling thread's current context; 0 when there is none yet.
cudaError_t current_context_id(unsigned long long *id) {
  static CtxGetCurrentFn get_current = nullptr;
  static CtxGetIdFn get_id = nullptr;
  if (!get_current || !get_id) {
    void *f1 = nullptr, *f2 = nullptr;
    cudaDriverEntryPointQueryResult q1, q2;
    cudaError_t e = cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000,
                                                     cudaEnableDefault, &q1);
    if (e != cudaSuccess || q1 != cudaDriverEntryPointSuccess) return cudaErrorNotSupported;
    e = cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2);
    if (e != cudaSuccess || q2 != cudaDriverEntryPointSuccess) return cudaErrorNotSupported;
    get_current = reinterpret_cast<CtxGetCurrentFn>(f1);
    get_id = reinterpret_cast<CtxGetIdFn>(f2);
  }
  CUcontext ctx = nullptr;
  if (get_current(&ctx) != CUDA_SUCCESS) return cudaErrorDeviceUninitialized;
  *id = 0;
  if (ctx && get_id(ctx, id) != CUDA_SUCCESS) return cudaErrorDeviceUninitialized;
  return cudaSuccess;
}

__device__ __forceinline__ double det3(const double J[3][3]) {
  return J[0][0] * J[1][1] * J[2][2] - J[0][0] * J[1][2] * J[2][1] -
         J[0][1] * J[1][0] * J[2][2] + J[0][1] * J[1][2] * J[2][0] +
         J[0][2] * J[1][0] * J[2][1] - J[0][2] * J[1][1] * J[2][0];
}

// Element volume from the interleaved node coordinates and the
// element-major connectivity: the same Jacobian, determinant and weights as
// the step's geometry phase.
__global__ void k_noalloc_elem_vol(const double *xyz, const int32_t *elnod, int64_t ne, int npe,
                                   double *vol) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ne) return;
  double x2[8][3];
  for (int a = 0; a < npe; a++) {
    const int64_t n = elnod[e * npe + a];
    x2[a][0] = xyz[3 * n];
    x2[a][1] = xyz[3 * n + 1];
    x2[a][2] = xyz[3 * n + 2];
  }
  double J[3][3];
  double w;
  if (npe == 8) {
    for (int k = 0; k < 3; k++) {
      J[0][k] = 0.125 * (-x2[0][k] + x2[1][k] + x2[2][k] - x2[3][k] - x2[4][k] + x2[5][k] +
                         x2[6][k] - x2[7][k]);
      J[1][k] = 0.125 * (-x2[0][k] - x2[1][k] + x2[2][k] + x2[3][k] - x2[4][k] - x2[5][k] +
                         x2[6][k] + x2[7][k]);
      J[2][k] = 0.125 * (-x2[0][k] - x2[1][k] - x2[2][k] - x2[3][k] + x2[4][k] + x2[5][k] +
                         x2[6][k] + x2[7][k]);
    }
    w = 8.0;
  } else {
    for (int k = 0; k < 3; k++) {
      J[0][k] = x2[1][k] - x2[0][k];
      J[1][k] = x2[2][k] - x2[0][k];
      J[2][k] = x2[3][k] - x2[0][k];
    }
    w = 1.0 / 6.0;
  }
  double v = 0.0;
  v += det3(J) * w * 1.0;
  vol[e] = v;
}

// Per-node sum of the volumes of the node's elements, in list order,
// divided by the nodes per element.
__global__ void k_noalloc_nodal_vol(const int32_t *offset, const int32_t *count,
                                    const int32_t *nodel, int64_t nn, int npe, const double *vol,
                                    double *voln) {
  const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= nn) return;
  const int32_t b = offset[n], c = count[n];
  double s = 0.0;
  for (int32_t k = 0; k < c; k++) s += vol[nodel[b + k]];
  s /= npe;
  voln[n] = s;
}

// Resolves the device address of the scratch array for the current device:
// once per device, again when that device's context has changed.
cudaError_t scratch_for_current_device(double **out) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  unsigned long long ctx = 0;
  e = current_context_id(&ctx);
  if (e != cudaSuccess) return e;
  ScratchAddr &a = g_scratch_addr[dev];
  if (!a.ptr || ctx == 0 || ctx != a.ctx_id) {
    void *p = nullptr;
    // also makes the device's primary context current when none was yet
    e = cudaGetSymbolAddress(&p, g_vol_scratch);
    if (e != cudaSuccess) return e;
    e = current_context_id(&ctx);
    if (e != cudaSuccess) return e;
    a.ptr = static_cast<double *>(p);
    a.ctx_id = ctx;
  }
  *out = a.ptr;
  return cudaSuccess;
}

}  // namespace

WF_API wf_status wf_nodal_volumes_noalloc(const double *xyz, const int32_t *elnod, int64_t nn,
                                          int64_t ne, int32_t npe, const int32_t *nodel_offset,
                                          const int32_t *nodel_count, const int32_t *nodel,
                                          double *voln, void *stream) {
  if (!xyz || !elnod || !nodel_offset || !nodel_count || !nodel || !voln) return WF_ERR_ARG;
  if (nn <= 0 || ne <= 0 || (npe != 8 && npe != 4)) return WF_ERR_ARG;
  if (ne > (int64_t)WF_NOALLOC_MAX_ELEMS) return WF_ERR_UNSUPPORTED;
  double *scratch = nullptr;
  if (scratch_for_current_device(&scratch) != cudaSuccess) return WF_ERR_CUDA;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  // a launch error of this call is reported and cleared; an error the
  // calling thread already had pending is left pending for its owner
  const cudaError_t before = cudaPeekAtLastError();
  k_noalloc_elem_vol<<<(unsigned)((ne + kThreads - 1) / kThreads), kThreads, 0, st>>>(
      xyz, elnod, ne, npe, scratch);
  cudaError_t after = cudaPeekAtLastError();
  if (after == before)
    k_noalloc_nodal_vol<<<(unsigned)((nn + kThreads - 1) / kThreads), kThreads, 0, st>>>(
        nodel_offset, nodel_count, nodel, nn, npe, scratch, voln);
  after = cudaPeekAtLastError();
  if (after == before) return WF_OK;
  if (before == cudaSuccess) cudaGetLastError();
  return WF_ERR_CUDA;
}
