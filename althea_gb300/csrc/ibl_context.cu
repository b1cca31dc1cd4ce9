// ibl_context.cu -- the bake context of include/althea_ibl.h: the GB300
// counterpart of ImageBasedLighting::createResources / precomputeResources
// (Src/ImageBasedLighting.cpp:137-412,415-605).  The env map stays resident
// on the device with its full mip chain; a bake writes irradiance, every
// prefiltered mip and (optionally) the BRDF LUT into caller-owned buffers,
// stream ordered, with no host synchronisation (the reference blocks on
// vkQueueWaitIdle, Src/SingleTimeCommandBuffer.cpp:28-54).
#include <cuda_runtime.h>

#include <cstring>
#include <new>
#include <string>

#include "althea_ibl.h"
#include "ibl_internal.h"

using namespace ibl;

struct althea_ibl_context {
  althea_ibl_config cfg;
  int device;
  int irr_w, irr_h;
  int mip_w[ALTHEA_IBL_MAX_MIPS], mip_h[ALTHEA_IBL_MAX_MIPS];
  float mip_r[ALTHEA_IBL_MAX_MIPS];
  float* chain;
  size_t chain_texels;
  void* irr_ws;          // plain path: irradiance partial sums
  size_t irr_ws_bytes;
  void* tc_ws;           // precision path: the planned contraction's workspace
  size_t tc_ws_bytes;
  bool env_ready;
  // Side streams for work independent of the tensor-core contractions: the
  // LUT (lut_side) and the outputs summed on the CUDA cores (narrow_side),
  // forked from and joined back into the caller's stream inside each bake.
  cudaStream_t lut_stream, narrow_stream;
  cudaEvent_t lut_fork, lut_join, narrow_fork, narrow_join;
  // Precision path: the workspace's direction tables and windows depend on
  // the sizes only, so the first bake computes them and `tables_done` (an
  // event after that bake) orders every later bake, on any stream, after it.
  bool tables_ready;
  cudaEvent_t tables_done;
  // Precision path: timing events around the contraction launch of the last
  // kTimedBakes bakes (bake i uses pair i % kTimedBakes), read by
  // althea_ibl_contraction_times.
  cudaEvent_t timing[ALTHEA_IBL_TIMED_BAKES][2];
  long long timed_bakes;
};

static void free_side_streams(althea_ibl_context* c) {
  if (c->lut_stream) cudaStreamDestroy(c->lut_stream);
  if (c->narrow_stream) cudaStreamDestroy(c->narrow_stream);
  for (cudaEvent_t ev : {c->lut_fork, c->lut_join, c->narrow_fork, c->narrow_join,
                         c->tables_done})
    if (ev) cudaEventDestroy(ev);
  for (auto& pair : c->timing)
    for (cudaEvent_t ev : pair)
      if (ev) cudaEventDestroy(ev);
}

static cudaError_t make_side_streams(althea_ibl_context* c) {
  cudaError_t e = cudaStreamCreateWithFlags(&c->lut_stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->narrow_stream, cudaStreamNonBlocking);
  for (cudaEvent_t* ev : {&c->lut_fork, &c->lut_join, &c->narrow_fork, &c->narrow_join,
                          &c->tables_done})
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(ev, cudaEventDisableTiming);
  if (c->cfg.path == ALTHEA_IBL_PATH_PRECISION)
    for (auto& pair : c->timing)
      for (cudaEvent_t& ev : pair)
        if (e == cudaSuccess) e = cudaEventCreate(&ev);
  return e;
}

// The context's mips as planner targets (no output pointers: planning and
// workspace sizing look at sizes and roughness only).
static void mip_targets(const althea_ibl_context* c, althea_ibl_mip_target* t) {
  const size_t texel = c->cfg.out_format == ALTHEA_IBL_FORMAT_RGBA16F ? 8 : 16;
  for (int m = 0; m < c->cfg.mip_count; ++m) {
    t[m].out_dev = nullptr;
    t[m].pitch_bytes = (size_t)c->mip_w[m] * texel;
    t[m].width = c->mip_w[m];
    t[m].height = c->mip_h[m];
    t[m].roughness = c->mip_r[m];
  }
}

extern "C" void althea_ibl_config_reference(althea_ibl_config* c, int w, int h) {
  if (!c) return;
  memset(c, 0, sizeof(*c));
  c->env_width = w;
  c->env_height = h;
  c->irradiance_width = w;   // Src/ImageBasedLighting.cpp:208-210
  c->irradiance_height = h;
  c->mip_count = 5;          // :184,192
  c->first_mip_width = w >> 1;
  c->first_mip_height = h >> 1;
  c->samples = 10000;        // PreFilterEnvMap.comp:5
  c->generator = ALTHEA_IBL_GEN_REF_HASH;
  c->lut_size = 0;           // the reference loads brdf_lut.png instead
  c->lut_samples = 1024;
  c->lut_orientation = ALTHEA_IBL_LUT_ASSET;
  c->path = ALTHEA_IBL_PATH_PLAIN;  // the reference's estimator
  c->out_format = ALTHEA_IBL_FORMAT_RGBA32F;
}

extern "C" int althea_ibl_create(const althea_ibl_config* cfg, althea_ibl_context** out) {
  if (!cfg || !out) return set_error(ALTHEA_IBL_ERR_INVALID_ARGUMENT, "null argument");
  *out = nullptr;
  int st = check_env(cfg->env_width, cfg->env_height);
  if (st) return st;
  althea_ibl_context* c = new (std::nothrow) althea_ibl_context();
  if (!c) return set_error(ALTHEA_IBL_ERR_OUT_OF_MEMORY, "host allocation");
  c->cfg = *cfg;
  const int w = cfg->env_width, h = cfg->env_height;
  c->irr_w = cfg->irradiance_width > 0 ? cfg->irradiance_width : w;
  c->irr_h = cfg->irradiance_height > 0 ? cfg->irradiance_height : h;
  if (cfg->mip_count < 1 || cfg->mip_count > ALTHEA_IBL_MAX_MIPS) {
    delete c;
    return set_error(ALTHEA_IBL_ERR_INVALID_ARGUMENT, "mip_count %d outside 1..%d",
                     cfg->mip_count, ALTHEA_IBL_MAX_MIPS);
  }
  int fw = cfg->first_mip_width > 0 ? cfg->first_mip_width : (w >> 1);
  int fh = cfg->first_mip_height > 0 ? cfg->first_mip_height : (h >> 1);
  if (fw < 1) fw = 1;
  if (fh < 1) fh = 1;
  for (int m = 0; m < cfg->mip_count; ++m) {
    c->mip_w[m] = (fw >> m) < 1 ? 1 : (fw >> m);
    c->mip_h[m] = (fh >> m) < 1 ? 1 : (fh >> m);
    // static_cast<float>(i) / 4.0f for 5 mips (Src/ImageBasedLighting.cpp:383)
    c->mip_r[m] = cfg->mip_count > 1 ? (float)m / (float)(cfg->mip_count - 1) : 0.0f;
  }
  if (cfg->samples < 1 || cfg->samples > (1 << 24) ||
      (cfg->generator != ALTHEA_IBL_GEN_REF_HASH && cfg->generator != ALTHEA_IBL_GEN_HAMMERSLEY)) {
    delete c;
    return set_error(ALTHEA_IBL_ERR_INVALID_ARGUMENT, "samples/generator");
  }
  if (cfg->lut_size < 0 || cfg->lut_size > 16384 ||
      (cfg->lut_size > 0 &&
       (cfg->lut_samples < 1 || cfg->lut_samples > (1 << 24) ||
        (cfg->lut_orientation != ALTHEA_IBL_LUT_ASSET &&
         cfg->lut_orientation != ALTHEA_IBL_LUT_CORRECTED)))) {
    delete c;
    return set_error(ALTHEA_IBL_ERR_INVALID_ARGUMENT, "lut_size/lut_samples/lut_orientation");
  }
  if (cfg->path != ALTHEA_IBL_PATH_PLAIN && cfg->path != ALTHEA_IBL_PATH_PRECISION) {
    delete c;
    return set_error(ALTHEA_IBL_ERR_INVALID_ARGUMENT, "path %d (plain 0, precision 1)",
                     cfg->path);
  }
  if (cfg->out_format != ALTHEA_IBL_FORMAT_RGBA32F &&
      cfg->out_format != ALTHEA_IBL_FORMAT_RGBA16F) {
    delete c;
    return set_error(ALTHEA_IBL_ERR_INVALID_ARGUMENT, "out_format %d (RGBA32F 0, RGBA16F 1)",
                     cfg->out_format);
  }
  if (cfg->path == ALTHEA_IBL_PATH_PLAIN && cfg->out_format != ALTHEA_IBL_FORMAT_RGBA32F) {
    delete c;
    return set_error(ALTHEA_IBL_ERR_UNSUPPORTED,
                     "out_format RGBA16F: the plain path writes RGBA32F (the reference's format)");
  }
  st = check_irradiance_args(w, h, c->irr_w, c->irr_h);
  if (st) {
    delete c;
    return st;
  }
  const bool precision = cfg->path == ALTHEA_IBL_PATH_PRECISION;
  if (precision) {
    // Plan now, so that a shape the planner cannot run is refused at create
    // and the workspace is sized once (the reference allocates its bake
    // temporaries per bake, Src/ImageBasedLighting.cpp:137-412).
    althea_ibl_mip_target t[ALTHEA_IBL_MAX_MIPS];
    mip_targets(c, t);
    c->tc_ws_bytes = tc_workspace_bytes(w, h, t, cfg->mip_count, nullptr, c->irr_w, c->irr_h, -1);
    if (c->tc_ws_bytes == 0) {
      delete c;
      const std::string why = last_error();  // set_error writes the same buffer
      return set_error(ALTHEA_IBL_ERR_UNSUPPORTED, "precision path: %s", why.c_str());
    }
  }
  cudaError_t e = cudaGetDevice(&c->device);
  if (e != cudaSuccess) {
    delete c;
    return cuda_status(e, "cudaGetDevice");
  }
  c->chain_texels = althea_ibl_chain_texels(w, h);
  if (!precision) c->irr_ws_bytes = irr_plan(w, h, c->irr_w, c->irr_h).workspace;
  e = cudaMalloc(&c->chain, c->chain_texels * 16);
  if (e == cudaSuccess && c->irr_ws_bytes) e = cudaMalloc(&c->irr_ws, c->irr_ws_bytes);
  if (e == cudaSuccess && c->tc_ws_bytes) e = cudaMalloc(&c->tc_ws, c->tc_ws_bytes);
  if (e == cudaSuccess) e = make_side_streams(c);
  if (e != cudaSuccess) {
    if (c->chain) cudaFree(c->chain);
    if (c->irr_ws) cudaFree(c->irr_ws);
    if (c->tc_ws) cudaFree(c->tc_ws);
    free_side_streams(c);
    delete c;
    return cuda_status(e, "context allocation");
  }
  *out = c;
  return ALTHEA_IBL_OK;
}

// The context's buffers live on the device that was current at create; a
// launch from another device would touch memory it may not reach.
static int check_device(const althea_ibl_context* c) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_status(e, "cudaGetDevice");
  if (dev != c->device)
    return set_error(ALTHEA_IBL_ERR_INVALID_ARGUMENT,
                     "the context lives on device %d but device %d is current", c->device, dev);
  return ALTHEA_IBL_OK;
}

extern "C" int althea_ibl_destroy(althea_ibl_context* c) {
  if (!c) return ALTHEA_IBL_OK;
  cudaFree(c->chain);
  if (c->irr_ws) cudaFree(c->irr_ws);
  if (c->tc_ws) cudaFree(c->tc_ws);
  free_side_streams(c);
  delete c;
  return ALTHEA_IBL_OK;
}

extern "C" int althea_ibl_mip_info(const althea_ibl_context* c, int m, int* w, int* h, float* r) {
  if (!c || m < 0 || m >= c->cfg.mip_count)
    return set_error(ALTHEA_IBL_ERR_INVALID_ARGUMENT, "mip index");
  if (w) *w = c->mip_w[m];
  if (h) *h = c->mip_h[m];
  if (r) *r = c->mip_r[m];
  return ALTHEA_IBL_OK;
}

extern "C" int althea_ibl_irradiance_size(const althea_ibl_context* c, int* w, int* h) {
  if (!c) return set_error(ALTHEA_IBL_ERR_INVALID_ARGUMENT, "null context");
  if (w) *w = c->irr_w;
  if (h) *h = c->irr_h;
  return ALTHEA_IBL_OK;
}

extern "C" const float* althea_ibl_env_chain(const althea_ibl_context* c) {
  return c ? c->chain : nullptr;
}

extern "C" int althea_ibl_upload_env(althea_ibl_context* c, const float* rgba, int src_is_device,
                                     void* stream) {
  ibl::NvtxRange nvtx_range("althea_ibl_upload_env");
  if (!c || !rgba) return set_error(ALTHEA_IBL_ERR_INVALID_ARGUMENT, "null argument");
  int r = check_device(c);
  if (r) return r;
  cudaStream_t st = (cudaStream_t)stream;
  size_t bytes = (size_t)c->cfg.env_width * c->cfg.env_height * 16;
  cudaError_t e = cudaMemcpyAsync(c->chain, rgba, bytes,
                                  src_is_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                                  st);
  if (e != cudaSuccess) return cuda_status(e, "env upload");
  r = launch_build_chain(c->chain, c->cfg.env_width, c->cfg.env_height, c->chain, st);
  if (r == ALTHEA_IBL_OK) c->env_ready = true;
  return r;
}

extern "C" int althea_ibl_bake(althea_ibl_context* c, const althea_ibl_outputs* o, void* stream) {
  ibl::NvtxRange nvtx_range("althea_ibl_bake");
  if (!c || !o) return set_error(ALTHEA_IBL_ERR_INVALID_ARGUMENT, "null argument");
  if (!c->env_ready)
    return set_error(ALTHEA_IBL_ERR_NOT_READY, "no environment map uploaded to this context");
  int r = check_device(c);
  if (r) return r;
  cudaStream_t st = (cudaStream_t)stream;
  const int w = c->cfg.env_width, h = c->cfg.env_height;
  const size_t texel = c->cfg.out_format == ALTHEA_IBL_FORMAT_RGBA16F ? 8 : 16;
  r = check_image(o->irradiance_dev, c->irr_w, c->irr_h, o->irradiance_pitch_bytes, texel,
                  "irradiance");
  if (r) return r;
  althea_ibl_mip_target mips[ALTHEA_IBL_MAX_MIPS];
  mip_targets(c, mips);
  for (int m = 0; m < c->cfg.mip_count; ++m) {
    mips[m].out_dev = o->mip_dev[m];
    mips[m].pitch_bytes = o->mip_pitch_bytes[m];
    r = check_image(mips[m].out_dev, mips[m].width, mips[m].height, mips[m].pitch_bytes, texel,
                    "prefiltered mip");
    if (r) return r;
  }
  if (c->cfg.lut_size > 0) {
    r = check_image(o->lut_dev, c->cfg.lut_size, c->cfg.lut_size, o->lut_pitch_bytes, 8, "lut");
    if (r) return r;
  }
  // The LUT does not depend on the env map: on the precision path it runs on
  // a side stream, beside the tensor-bound contractions, and is joined below.
  const bool precision = c->cfg.path == ALTHEA_IBL_PATH_PRECISION;
  const bool lut_side = precision && c->cfg.lut_size > 0;
  if (lut_side) {
    cudaError_t e = cudaEventRecord(c->lut_fork, st);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(c->lut_stream, c->lut_fork, 0);
    if (e != cudaSuccess) return cuda_status(e, "LUT side-stream fork");
    r = launch_brdf_lut(o->lut_dev, c->cfg.lut_size, o->lut_pitch_bytes, c->cfg.lut_samples,
                        c->cfg.lut_orientation, c->lut_stream);
    if (r) return r;
    e = cudaEventRecord(c->lut_join, c->lut_stream);
    if (e != cudaSuccess) return cuda_status(e, "LUT side-stream record");
  }
  if (precision) {
    // the planner's source levels (-1), the workspace sized at create
    const SideStream side{c->narrow_stream, c->narrow_fork, c->narrow_join};
    if (c->tables_ready) {
      const cudaError_t e = cudaStreamWaitEvent(st, c->tables_done, 0);
      if (e != cudaSuccess) r = cuda_status(e, "tables event wait");
    }
    if (!r)
      r = tc_bake(c->chain, w, h, mips, c->cfg.mip_count, nullptr, o->irradiance_dev, c->irr_w,
                  c->irr_h, o->irradiance_pitch_bytes, -1, c->tc_ws, c->tc_ws_bytes,
                  c->cfg.out_format, st, &side, !c->tables_ready,
                  c->timing[c->timed_bakes % ALTHEA_IBL_TIMED_BAKES]);
    if (!r) ++c->timed_bakes;
    if (!r && !c->tables_ready) {
      const cudaError_t e = cudaEventRecord(c->tables_done, st);
      if (e == cudaSuccess)
        c->tables_ready = true;
      else
        r = cuda_status(e, "tables event record");
    }
    if (lut_side) {  // join even when the bake failed, so no fork is left open
      const cudaError_t e = cudaStreamWaitEvent(st, c->lut_join, 0);
      if (!r && e != cudaSuccess) r = cuda_status(e, "LUT side-stream join");
    }
    return r;
  } else {
    // Src/ImageBasedLighting.cpp:315-343: irradiance dispatch; :353-395: one
    // prefilter dispatch per mip (here one launch for the whole chain).
    r = launch_prefilter(c->chain, w, h, mips, c->cfg.mip_count, c->cfg.samples,
                         c->cfg.generator, st);
    if (r) return r;
    r = launch_irradiance(c->chain, w, h, o->irradiance_dev, c->irr_w, c->irr_h,
                          o->irradiance_pitch_bytes, c->irr_ws, st);
    if (r) return r;
  }
  if (c->cfg.lut_size > 0)
    r = launch_brdf_lut(o->lut_dev, c->cfg.lut_size, o->lut_pitch_bytes, c->cfg.lut_samples,
                        c->cfg.lut_orientation, st);
  return r;
}

extern "C" int althea_ibl_bake_status(const althea_ibl_context* c, void* stream) {
  if (!c) return set_error(ALTHEA_IBL_ERR_INVALID_ARGUMENT, "null context");
  int r = check_device(c);
  if (r) return r;
  if (c->cfg.path == ALTHEA_IBL_PATH_PRECISION) return althea_ibl_tc_error(c->tc_ws, stream);
  return cuda_status(cudaStreamSynchronize((cudaStream_t)stream), "bake status");
}

extern "C" int althea_ibl_contraction_times(const althea_ibl_context* c, float* ms,
                                            int max_count, int* count) {
  if (!c || !count || max_count < 0 || (max_count > 0 && !ms))
    return set_error(ALTHEA_IBL_ERR_INVALID_ARGUMENT, "contraction times: null or negative");
  *count = 0;
  if (c->cfg.path != ALTHEA_IBL_PATH_PRECISION)
    return set_error(ALTHEA_IBL_ERR_UNSUPPORTED, "contraction times: plain-path context");
  int r = check_device(c);
  if (r) return r;
  long long n = c->timed_bakes < ALTHEA_IBL_TIMED_BAKES ? c->timed_bakes : ALTHEA_IBL_TIMED_BAKES;
  if (n > max_count) n = max_count;
  for (long long k = 0; k < n; ++k) {  // oldest first
    const cudaEvent_t* pair = c->timing[(c->timed_bakes - n + k) % ALTHEA_IBL_TIMED_BAKES];
    cudaError_t e = cudaEventSynchronize(pair[1]);
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms[k], pair[0], pair[1]);
    if (e != cudaSuccess) return cuda_status(e, "contraction times");
  }
  *count = (int)n;
  return ALTHEA_IBL_OK;
}

extern "C" size_t althea_ibl_context_device_bytes(const althea_ibl_context* c) {
  if (!c) return 0;
  return c->chain_texels * 16 + c->irr_ws_bytes + c->tc_ws_bytes;
}
