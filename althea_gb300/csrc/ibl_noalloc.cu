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
// The array costs ALTHEA_IBL_NOALLOC_SCRATCH_BYTES of device memory on every
// GPU that loads the library, until the process exits.  All calls share it:
// two calls whose kernels overlap on the GPU (different streams, or
// different host threads) race on it and must be serialised by the caller.
// Nothing in it needs clearing between calls: a call reads only partial sums
// that the same call wrote earlier on the same stream.
#include <cuda_runtime.h>

#include <mutex>

#include "althea_ibl.h"
#include "ibl_internal.h"

namespace {

static __device__ __align__(256) unsigned char g_irradiance_scratch[ALTHEA_IBL_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
void* g_scratch_ptr[kMaxDevices] = {};

// The symbol's name is only a host-side stand-in; the device address must be
// asked for once per device with that device current.
int scratch_for_current_device(void** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return ibl::cuda_status(e, "cudaGetDevice");
  if (dev < 0 || dev >= kMaxDevices)
    return ibl::set_error(ALTHEA_IBL_ERR_UNSUPPORTED, "device ordinal %d >= %d", dev,
                          kMaxDevices);
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_irradiance_scratch);
    if (e != cudaSuccess) return ibl::cuda_status(e, "cudaGetSymbolAddress(irradiance scratch)");
    g_scratch_ptr[dev] = p;
  }
  *out = g_scratch_ptr[dev];
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
  st = scratch_for_current_device(&scratch);
  if (st) return st;
  return ibl::launch_irradiance(chain, w, h, out, ow, oh, pitch, scratch, (cudaStream_t)stream);
}
