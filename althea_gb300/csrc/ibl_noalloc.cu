// ibl_noalloc.cu -- irradiance without any device allocation.
//
// Some callers cannot call cudaMalloc: a renderer that hands every byte of
// device memory out through its own allocator and budget (the way the
// reference engine owns all GPU memory through its VMA-based allocator), a
// plug-in that is given a fixed memory envelope, or code that runs inside a
// frame or a real-time callback where an allocation may stall the device.
// For them this entry point runs the same irradiance kernels as
// althea_ibl_irradiance, but keeps the per-block partial sums in a fixed
// array that lives in the library image itself, so the caller passes only
// the chain and the output.
//
// The array costs ALTHEA_IBL_NOALLOC_SCRATCH_BYTES of device memory in every
// CUDA context that loads this module, until the context is destroyed or the
// process exits.  With lazy module loading (CUDA_MODULE_LOADING=LAZY, the
// default) the module, and so the array, is loaded by the first call in a
// context: that first call commits the memory and should be made once as a
// warm-up, outside any frame loop and before any stream capture.  All calls
// in one context share the array: two calls whose kernels overlap on the GPU
// (different streams, or different host threads) race on it and must be
// serialised by the caller.  The batch and server entry points never use it.
// Nothing in it needs clearing between calls: a call reads only partial sums
// that the same call wrote earlier on the same stream.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <mutex>

#include "althea_ibl.h"
#include "ibl_internal.h"

namespace {

static __device__ __align__(256) unsigned char g_irradiance_scratch[ALTHEA_IBL_NOALLOC_SCRATCH_BYTES];

// The symbol's name is only a host-side stand-in; its device address belongs
// to the CUDA context that loaded the module.  It is looked up once per
// context, with that context current, and cached under the context's unique
// id (cuCtxGetId), not under the device ordinal: a caller may make its own
// driver-API context current, and cudaDeviceReset replaces the primary
// context (the new one has a new id, so the lookup runs again).  The driver
// calls are reached through cudaGetDriverEntryPointByVersion, so the library
// does not link libcuda.
constexpr int kMaxContexts = 64;
std::mutex g_setup_mutex;
struct ScratchEntry {
  unsigned long long ctx_id;
  void* ptr;
};
ScratchEntry g_scratch[kMaxContexts] = {};
int g_scratch_count = 0;
PFN_cuCtxGetCurrent_v4000 g_ctx_get_current = nullptr;
PFN_cuCtxGetId_v12000 g_ctx_get_id = nullptr;

int resolve_driver_calls() {
  if (g_ctx_get_current && g_ctx_get_id) return ALTHEA_IBL_OK;
  cudaDriverEntryPointQueryResult q1 = cudaDriverEntryPointSymbolNotFound, q2 = q1;
  void *f1 = nullptr, *f2 = nullptr;
  cudaError_t e = cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 4000, cudaEnableDefault,
                                                   &q1);
  if (e == cudaSuccess)
    e = cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2);
  if (e != cudaSuccess) return ibl::cuda_status(e, "cudaGetDriverEntryPointByVersion");
  if (q1 != cudaDriverEntryPointSuccess || q2 != cudaDriverEntryPointSuccess || !f1 || !f2)
    return ibl::set_error(ALTHEA_IBL_ERR_CUDA,
                          "the driver does not provide cuCtxGetCurrent / cuCtxGetId");
  g_ctx_get_current = reinterpret_cast<PFN_cuCtxGetCurrent_v4000>(f1);
  g_ctx_get_id = reinterpret_cast<PFN_cuCtxGetId_v12000>(f2);
  return ALTHEA_IBL_OK;
}

int scratch_for_current_context(void** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return ibl::cuda_status(e, "cudaGetDevice");
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  int st = resolve_driver_calls();
  if (st) return st;
  CUcontext ctx = nullptr;
  if (g_ctx_get_current(&ctx) != CUDA_SUCCESS || !ctx) {
    // No context current on this thread yet: cudaSetDevice makes the
    // device's primary context current (the lookup below needs one).
    e = cudaSetDevice(dev);
    if (e != cudaSuccess) return ibl::cuda_status(e, "cudaSetDevice");
    if (g_ctx_get_current(&ctx) != CUDA_SUCCESS || !ctx)
      return ibl::set_error(ALTHEA_IBL_ERR_CUDA, "no CUDA context current on device %d", dev);
  }
  unsigned long long id = 0;
  if (g_ctx_get_id(ctx, &id) != CUDA_SUCCESS)
    return ibl::set_error(ALTHEA_IBL_ERR_CUDA, "cuCtxGetId failed on device %d", dev);
  for (int k = 0; k < g_scratch_count; ++k)
    if (g_scratch[k].ctx_id == id) {
      *out = g_scratch[k].ptr;
      return ALTHEA_IBL_OK;
    }
  void* p = nullptr;
  e = cudaGetSymbolAddress(&p, g_irradiance_scratch);
  if (e != cudaSuccess) return ibl::cuda_status(e, "cudaGetSymbolAddress(irradiance scratch)");
  // Remember it; when the table is full the oldest entry gives way (its
  // context is most likely gone).
  if (g_scratch_count < kMaxContexts) {
    g_scratch[g_scratch_count++] = ScratchEntry{id, p};
  } else {
    for (int k = 1; k < kMaxContexts; ++k) g_scratch[k - 1] = g_scratch[k];
    g_scratch[kMaxContexts - 1] = ScratchEntry{id, p};
  }
  *out = p;
  return ALTHEA_IBL_OK;
}

}  // namespace

extern "C" int althea_ibl_irradiance_noalloc(const float* chain, int w, int h, float* out,
                                             int ow, int oh, size_t pitch, void* stream) {
  int st = ibl::check_env(w, h);
  if (st) return st;
  st = ibl::check_irradiance_args(w, h, ow, oh);
  if (st) return st;
  if (!chain || ((uintptr_t)chain) % 16)
    return ibl::set_error(ALTHEA_IBL_ERR_INVALID_ARGUMENT, "chain: null or not 16-byte aligned");
  st = ibl::check_image(out, ow, oh, pitch, 16, "irradiance");
  if (st) return st;
  ibl::IrrPlan pl = ibl::irr_plan(w, h, ow, oh);
  if (pl.workspace > (size_t)ALTHEA_IBL_NOALLOC_SCRATCH_BYTES)
    return ibl::set_error(ALTHEA_IBL_ERR_UNSUPPORTED,
                          "irradiance %dx%d needs %zu bytes of partial sums; the no-allocation "
                          "variant holds at most %d (use althea_ibl_irradiance with a workspace)",
                          ow, oh, pl.workspace, ALTHEA_IBL_NOALLOC_SCRATCH_BYTES);
  void* scratch = nullptr;
  st = scratch_for_current_context(&scratch);
  if (st) return st;
  return ibl::launch_irradiance(chain, w, h, out, ow, oh, pitch, scratch, (cudaStream_t)stream);
}
