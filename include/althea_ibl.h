/*
 * althea_ibl.h -- C ABI of the GB300 image-based-lighting precompute.
 *
 * Drop-in for the IBL bake of the Althea engine: the reference records two
 * compute dispatches per bake inside
 *   ImageBasedLighting::precomputeResources   (Src/ImageBasedLighting.cpp:137-412)
 * reached from
 *   ImageBasedLighting::createResources       (Include/Althea/ImageBasedLighting.h:46-49,
 *                                              Src/ImageBasedLighting.cpp:415-605)
 * and binds env / prefiltered / irradiance / BRDF-LUT images in that order
 * (Src/ImageBasedLighting.cpp:20-26, Shaders/DeferredPass.frag:10-13).
 *
 * Conventions
 *  - Images are RGBA32F (float4 per texel) unless a format says otherwise,
 *    row-major with row 0 = v = 0, addressed with a row pitch in BYTES.
 *  - Every pointer named *_dev is CUDA device memory owned by the caller.
 *  - `stream` is a cudaStream_t passed as void* (NULL = legacy default
 *    stream).  All kernel entry points are asynchronous and stream ordered.
 *  - Every function returns althea_ibl_status.  No C++ exception crosses this
 *    boundary.  althea_ibl_last_error() returns the calling thread's last
 *    error message (the reference throws std::runtime_error instead,
 *    Src/ImageBasedLighting.cpp:423-425).
 */
#ifndef ALTHEA_IBL_H
#define ALTHEA_IBL_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ALTHEA_IBL_ABI_VERSION 2   /* 2: config path/out_format, resident server maps, suns */
#define ALTHEA_IBL_MAX_LEVELS 16   /* env maps up to 32768 wide */
#define ALTHEA_IBL_MAX_MIPS 16     /* prefiltered chain length */

/* Bake path: the reference estimator (PreFilterEnvMap.comp /
 * GenIrradianceMap.comp, bit for bit) or the quadrature it estimates as a
 * tensor-core contraction within 1e-3 of FP64 (the precision path below). */
#define ALTHEA_IBL_PATH_PLAIN 0       /* the reference estimator */
#define ALTHEA_IBL_PATH_PRECISION 1   /* tensor-core contraction, <= 1e-3 vs FP64 */

/* Output formats of the prefiltered mips and the irradiance (the precision
 * path writes either; the plain path writes RGBA32F, the reference's format,
 * Src/ImageBasedLighting.cpp:156-166,192-221). */
#define ALTHEA_IBL_FORMAT_RGBA32F 0   /* 16-byte texels (VK_FORMAT_R32G32B32A32_SFLOAT) */
#define ALTHEA_IBL_FORMAT_RGBA16F 1   /* 8-byte texels (IEEE half), alpha 1
                                         (VK_FORMAT_R16G16B16A16_SFLOAT) */

typedef enum {
  ALTHEA_IBL_OK = 0,
  ALTHEA_IBL_ERR_INVALID_ARGUMENT = 1,
  ALTHEA_IBL_ERR_CUDA = 2,
  ALTHEA_IBL_ERR_OUT_OF_MEMORY = 3,
  ALTHEA_IBL_ERR_UNSUPPORTED = 4,
  ALTHEA_IBL_ERR_BUDGET = 5,
  ALTHEA_IBL_ERR_NOT_READY = 6
} althea_ibl_status;

/* Sample generator of the GGX prefilter.
 * REF_HASH: the ShaderToy integer hash of PreFilterEnvMap.comp:38-44 seeded
 *   with the texel position (:127), two draws per sample (:85) -- the
 *   reference estimator, bit for bit.
 * HAMMERSLEY: xi_i = (i/N, bitreverse(i) * 2^-32) in place of the two draws. */
typedef enum { ALTHEA_IBL_GEN_REF_HASH = 0, ALTHEA_IBL_GEN_HAMMERSLEY = 1 } althea_ibl_generator;

/* BRDF LUT row order.  ASSET: row 0 = roughness 1, the layout of the
 * reference's Content/PrecomputedMaps/brdf_lut.png that its renderer binds
 * today.  CORRECTED: row 0 = roughness 0, matching
 * texture(brdfLut, vec2(NdotV, roughness)) in Shaders/PBR/PBRMaterial.glsl:110. */
typedef enum { ALTHEA_IBL_LUT_ASSET = 0, ALTHEA_IBL_LUT_CORRECTED = 1 } althea_ibl_lut_orientation;

/* One prefiltered mip: replaces one dispatch of PreFilterEnvMap.comp with
 * push constants {envMapWidth, envMapHeight, width, height, roughness}
 * (PrefilterEnvMapPushConstants, Src/ImageBasedLighting.cpp:123-129,376-395). */
typedef struct {
  float* out_dev;      /* RGBA32F, width x height */
  size_t pitch_bytes;  /* >= width * 16, multiple of 16 */
  int width, height;
  float roughness;     /* reference: i / 4 for mip i of 5 */
} althea_ibl_mip_target;

/* ---- environment mip chain ------------------------------------------------
 * Replaces Image::generateMipMaps (Src/Image.cpp:135-239: vkCmdBlitImage with
 * VK_FILTER_LINEAR per level) for the RGBA32F env image created at
 * Src/ImageBasedLighting.cpp:156-166 with computeMipCount levels
 * (Src/Utilities.cpp:97-100).  The chain is every level back to back, level 0
 * first, tightly packed (row pitch = level width * 16 bytes). */
int althea_ibl_chain_levels(int env_width, int env_height);
size_t althea_ibl_chain_texels(int env_width, int env_height);
size_t althea_ibl_chain_level_offset(int env_width, int env_height, int level);
/* level0_dev may equal chain_dev (level 0 is then used in place). */
int althea_ibl_build_env_chain(const float* level0_dev, int env_width, int env_height,
                               float* chain_dev, void* stream);

/* ---- GGX prefilter (PreFilterEnvMap.comp:126-177) ----------------------------
 * All listed mips in one launch.  samples = MAX_SAMPLES of the shader (:5; the
 * reference uses 10000), also used by the source-LOD rule (:158). */
int althea_ibl_prefilter(const float* chain_dev, int env_width, int env_height,
                         const althea_ibl_mip_target* mips, int mip_count, int samples,
                         int generator, void* stream);

/* ---- diffuse irradiance (GenIrradianceMap.comp:106-155) -------------------
 * Output size is free (the reference dispatches it at env size,
 * Src/ImageBasedLighting.cpp:208-221,328-343); the 300 x int(300 H / W) grid
 * and the LOD log2(W / 300) come from the env size as in the shader.
 * Needs a caller-provided device workspace of
 * althea_ibl_irradiance_workspace_size() bytes for per-block partial sums. */
size_t althea_ibl_irradiance_workspace_size(int env_width, int env_height, int out_width,
                                            int out_height);
int althea_ibl_irradiance(const float* chain_dev, int env_width, int env_height, float* out_dev,
                          int out_width, int out_height, size_t out_pitch_bytes,
                          void* workspace_dev, size_t workspace_bytes, void* stream);

/* ---- irradiance without device allocation ---------------------------------
 * No counterpart in the reference: an addition for callers that cannot call
 * cudaMalloc (a renderer that owns all device memory through its own
 * allocator and budget, a plug-in with a fixed memory envelope, code inside a
 * frame or real-time callback where an allocation may stall the device).
 * Same kernels and results as althea_ibl_irradiance, but the partial sums
 * live in a fixed array of ALTHEA_IBL_NOALLOC_SCRATCH_BYTES inside the
 * library; the call allocates nothing.  Outputs whose partial sums do not fit
 * are rejected with ALTHEA_IBL_ERR_UNSUPPORTED: up to 262,144 output texels
 * (512 x 512, or 512 x 256) fit, 262,145 and more (1024 x 512) do not.
 * The array is device memory of the CUDA context current at the call, held
 * until that context is destroyed or the process exits.  With lazy module
 * loading (the CUDA default) it is committed by the first call in each
 * context, and that first call also looks up the array's device address
 * (once per context, cached under the context's id): make one warm-up call
 * outside any frame loop and before any stream capture.  All calls in a
 * context share the array: calls whose kernels overlap on the GPU (other
 * streams, other host threads) race on it and must be serialised by the
 * caller; the batch and server calls never use it. */
#define ALTHEA_IBL_NOALLOC_SCRATCH_BYTES (4 * 1024 * 1024)
int althea_ibl_irradiance_noalloc(const float* chain_dev, int env_width, int env_height,
                                  float* out_dev, int out_width, int out_height,
                                  size_t out_pitch_bytes, void* stream);

/* ---- split-sum BRDF LUT ----------------------------------------------------
 * Computes what the reference loads from Content/PrecomputedMaps/brdf_lut.png
 * (Src/ImageBasedLighting.cpp:570-603): RG32F n x n, R = scale, G = bias of
 * the split-sum integral (GGX alpha = roughness^2, Smith k = alpha/2,
 * Hammersley samples). */
int althea_ibl_brdf_lut(float* out_dev, int n, size_t pitch_bytes, int samples, int orientation,
                        void* stream);

/* ---- bake context: the createResources / precomputeResources mirror ------- */
typedef struct althea_ibl_context althea_ibl_context;

typedef struct {
  int env_width, env_height;      /* resident env map size */
  int irradiance_width, irradiance_height;   /* 0 = env size (reference) */
  int mip_count;                  /* prefiltered mips (reference: 5) */
  int first_mip_width, first_mip_height;     /* 0 = env size / 2 (reference) */
  int samples;                    /* reference: 10000 */
  int generator;                  /* althea_ibl_generator */
  int lut_size;                   /* 0 = no LUT */
  int lut_samples;
  int lut_orientation;            /* althea_ibl_lut_orientation */
  int path;                       /* ALTHEA_IBL_PATH_* (reference: PLAIN) */
  int out_format;                 /* ALTHEA_IBL_FORMAT_* of the mips and the irradiance
                                     (reference: RGBA32F; RGBA16F needs PATH_PRECISION) */
} althea_ibl_config;

/* Fills the reference's own settings for an env map of the given size. */
void althea_ibl_config_reference(althea_ibl_config* cfg, int env_width, int env_height);

typedef struct {
  float* irradiance_dev;
  size_t irradiance_pitch_bytes;
  float* mip_dev[ALTHEA_IBL_MAX_MIPS];
  size_t mip_pitch_bytes[ALTHEA_IBL_MAX_MIPS];
  float* lut_dev;                 /* RG32F; may be NULL when lut_size == 0 */
  size_t lut_pitch_bytes;
} althea_ibl_outputs;

/* The context's device memory lives on the device current at create;
 * upload_env and bake refuse to run while another device is current.
 * create refuses (ALTHEA_IBL_ERR_UNSUPPORTED) a precision config the planner
 * cannot run and RGBA16F outputs on the plain path. */
int althea_ibl_create(const althea_ibl_config* cfg, althea_ibl_context** out);
int althea_ibl_destroy(althea_ibl_context* ctx);
/* Mip m size and roughness as the context bakes them. */
int althea_ibl_mip_info(const althea_ibl_context* ctx, int mip, int* width, int* height,
                        float* roughness);
int althea_ibl_irradiance_size(const althea_ibl_context* ctx, int* width, int* height);
/* Uploads level 0 (host or device memory, RGBA32F, tightly packed) into the
 * context's resident chain and rebuilds the mip chain. */
int althea_ibl_upload_env(althea_ibl_context* ctx, const float* rgba, int src_is_device,
                          void* stream);
/* Resident chain (device), for callers that bind the env map itself. */
const float* althea_ibl_env_chain(const althea_ibl_context* ctx);
/* Irradiance + every prefiltered mip (+ LUT when configured) into caller
 * buffers: the dispatch sequence of Src/ImageBasedLighting.cpp:315-402.
 * With path = ALTHEA_IBL_PATH_PRECISION the context plans the contraction
 * (althea_ibl_tc_plan's source levels) and holds its workspace, sized at
 * create; the mips and the irradiance are then written in cfg.out_format
 * (the althea_ibl_outputs pointers point to texels of that format, pitches
 * in bytes).  The LUT is RG32F on both paths. */
int althea_ibl_bake(althea_ibl_context* ctx, const althea_ibl_outputs* outs, void* stream);
/* Synchronises the stream, then reports a precision bake whose kernels gave
 * up on a bounded wait (ALTHEA_IBL_ERR_CUDA); ALTHEA_IBL_OK otherwise and on
 * the plain path.  Replaces the reference's blocking vkQueueWaitIdle
 * (Src/SingleTimeCommandBuffer.cpp:28-54) for callers that want the result
 * checked. */
int althea_ibl_bake_status(const althea_ibl_context* ctx, void* stream);
/* Device time of the contraction launch (every tcgen05 contraction of a
 * bake, one launch) of the last min(bakes, ALTHEA_IBL_TIMED_BAKES, max_count)
 * precision bakes, oldest first, in ms: from timing events the context
 * records on the bake's stream around that launch.  Synchronises on those
 * events.  No counterpart in the reference (its bake is timed nowhere);
 * for rooflines and monitoring.  ALTHEA_IBL_ERR_UNSUPPORTED on the plain path. */
#define ALTHEA_IBL_TIMED_BAKES 64
int althea_ibl_contraction_times(const althea_ibl_context* ctx, float* ms, int max_count,
                                 int* count);
/* Device bytes the context holds (chain + workspaces), as allocated at create. */
size_t althea_ibl_context_device_bytes(const althea_ibl_context* ctx);

/* ---- precision path: dense contraction on the tensor cores -------------------
 * Replaces the two estimators of Shaders/IBL_Precompute (GenIrradianceMap.comp,
 * PreFilterEnvMap.comp) by the
 * quadrature they estimate: prefilter(n) = sum_t L_t w / sum_t w with
 * w = D_GGX(n.h) max(0, n.w_t) Omega_t, irradiance(n) = (1/pi) sum_t L_t
 * max(0, n.w_t) Omega_t, over the texels of one env level per output (picked
 * by althea_ibl_tc_plan so the result stays within 1e-3 of the same sum over
 * level 0; levels[m] = -1 selects the plan).  tcgen05 BF16 hi/lo MMAs with
 * FP32 accumulation in TMEM, FP64 weight normalisation.  Roughness-0 mips
 * (a delta) take the plain path.  Contracted outputs (mips of roughness > 0,
 * the irradiance) are at most 1024 wide, and their source level a whole
 * multiple of their width; other shapes are refused with
 * ALTHEA_IBL_ERR_UNSUPPORTED (althea_ibl_tc_workspace_size returns 0).
 * Workspace: althea_ibl_tc_workspace_size bytes, 256-byte aligned.
 * althea_ibl_tc_error synchronises the stream and reports a kernel that gave
 * up on a bounded wait. */
size_t althea_ibl_tc_workspace_size(int env_width, int env_height,
                                    const althea_ibl_mip_target* mips, int mip_count,
                                    const int* levels, int irradiance_width,
                                    int irradiance_height, int irradiance_level);
int althea_ibl_tc_plan(int env_width, int env_height, const althea_ibl_mip_target* mips,
                       int mip_count, int irradiance_width, int* levels_out,
                       int* irradiance_level_out);
int althea_ibl_bake_tc(const float* chain_dev, int env_width, int env_height,
                       const althea_ibl_mip_target* mips, int mip_count, const int* levels,
                       float* irradiance_dev, int irradiance_width, int irradiance_height,
                       size_t irradiance_pitch_bytes, int irradiance_level, void* workspace_dev,
                       size_t workspace_bytes, void* stream);
int althea_ibl_tc_error(const void* workspace_dev, void* stream);
/* The planned work of a precision bake, as its kernels run it (host only, no
 * device access): for benchmarks and rooflines.  No counterpart in the
 * reference. */
typedef struct {
  double dense_pairs;        /* (output texel, source texel) pairs of the tensor-core outputs */
  double visible_pairs;      /* of those, the pairs in the K stages the kernels run (the rest
                                lie below every row's horizon: exact zeros, skipped) */
  double tensor_flops;       /* flops of the tcgen05.mma instructions issued (M = 128 tiles,
                                padding rows and columns included) */
  double cuda_core_pairs;    /* pairs of the outputs summed on the CUDA cores */
  int tensor_launches;       /* contraction launches: 1 (every contraction of a bake runs
                                as work items of one queue launch) */
} althea_ibl_tc_work;
int althea_ibl_tc_stats(int env_width, int env_height, const althea_ibl_mip_target* mips,
                        int mip_count, const int* levels, int irradiance_width,
                        int irradiance_height, int irradiance_level, althea_ibl_tc_work* out);
/* Diagnostics: runs the precision kernel's bounded mbarrier wait on a barrier
 * that nothing completes, with a limit of limit_ns (1 ns .. 1 s).  Returns
 * ALTHEA_IBL_OK when the wait gave up, raised its abort flag and the kernel
 * returned (the context stays usable); *waited_ms = the time it waited.
 * Synchronises the stream. */
int althea_ibl_tc_wait_selftest(unsigned long long limit_ns, int* waited_ms, void* stream);

/* althea_ibl_bake_tc with the output format chosen (ALTHEA_IBL_FORMAT_*):
 * with RGBA16F, the images the renderer binds as
 * VK_FORMAT_R16G16B16A16_SFLOAT (the mips' out_dev and irradiance_dev then
 * point to RGBA16F texels; pitches in bytes). */
int althea_ibl_bake_tc_ex(const float* chain_dev, int env_width, int env_height,
                          const althea_ibl_mip_target* mips, int mip_count, const int* levels,
                          void* irradiance_dev, int irradiance_width, int irradiance_height,
                          size_t irradiance_pitch_bytes, int irradiance_level, void* workspace_dev,
                          size_t workspace_bytes, int out_format, void* stream);

/* ---- batched bakes -----------------------------------------------------------
 * No single counterpart in the reference, which bakes one probe per
 * createResources call (Src/GlobalResources.cpp:18-22); a batch bakes many
 * probes of uneven size and mip count as one CUDA-graph launch:
 *   env chains (one launch per level index over all probes), a persistent
 *   prefilter kernel draining a (probe, mip, tile) work queue, a batched
 *   irradiance and an optional shared LUT.
 * Results are identical to baking each probe alone with the stateless calls.
 * With ALTHEA_IBL_BATCH_AUTOTUNE the plan times its candidate tile shapes and
 * irradiance split factors once per batch shape and caches the choice (in
 * memory, and in the file named by $ALTHEA_IBL_TUNE_CACHE when set). */
typedef struct {
  const float* level0_dev;   /* env level 0; NULL if chain_dev already holds the chain */
  float* chain_dev;          /* althea_ibl_chain_texels(W, H) RGBA32F texels */
  int env_width, env_height;
  float* irradiance_dev;     /* may be NULL: no irradiance for this probe */
  int irradiance_width, irradiance_height;
  size_t irradiance_pitch_bytes;
  int mip_count;
  float* mip_dev[ALTHEA_IBL_MAX_MIPS];
  size_t mip_pitch_bytes[ALTHEA_IBL_MAX_MIPS];
  int mip_width[ALTHEA_IBL_MAX_MIPS], mip_height[ALTHEA_IBL_MAX_MIPS];
  float mip_roughness[ALTHEA_IBL_MAX_MIPS];
} althea_ibl_probe;

#define ALTHEA_IBL_BATCH_AUTOTUNE 1
#define ALTHEA_IBL_BATCH_GRAPH 2
/* Mips and irradiance by the precision path, after the shared chain pass:
 * every probe's split planes and tables, then ONE persistent tcgen05
 * contraction kernel draining a queue of (probe output, row tile, column
 * block, source split) work items of every probe, largest first, then every
 * probe's finish.  Each probe gets its own workspace of
 * althea_ibl_tc_workspace_size bytes.  Results are identical to
 * althea_ibl_bake_tc_ex of each probe alone (planner's levels); check them
 * with althea_ibl_batch_status. */
#define ALTHEA_IBL_BATCH_PRECISION 4
/* With ALTHEA_IBL_BATCH_PRECISION: RGBA16F outputs (8-byte texels). */
#define ALTHEA_IBL_BATCH_HALF 8

typedef struct {
  int samples;
  int generator;
  float* lut_dev;            /* shared RG32F LUT, or NULL */
  int lut_size;
  size_t lut_pitch_bytes;
  int lut_samples;
  int lut_orientation;
  int flags;                 /* ALTHEA_IBL_BATCH_* */
} althea_ibl_batch_params;

typedef struct {
  int probes, prefilter_jobs, prefilter_tiles, irradiance_blocks;
  int tile_x, tile_y;        /* prefilter tile chosen */
  int persistent_blocks;     /* prefilter grid */
  int irradiance_target_blocks;
  int tuned;                 /* 1 if the choice came from timing (now or cached) */
  int graph;                 /* 1 once the bake is a captured CUDA graph */
  int graph_kernels;         /* kernel launches in that graph (-1 before capture) */
  int contraction_items;     /* precision: work items of the persistent contraction */
} althea_ibl_batch_info;

typedef struct althea_ibl_batch althea_ibl_batch;

/* Builds the plan (copies the probe table to the device; autotunes when
 * asked, which runs the batch on `stream`).  Probe buffers must outlive it. */
int althea_ibl_batch_create(const althea_ibl_probe* probes, int n,
                            const althea_ibl_batch_params* params, void* stream,
                            althea_ibl_batch** out);
/* Bakes every probe (chains when level0_dev is set, mips, irradiance, LUT). */
int althea_ibl_batch_run(althea_ibl_batch* batch, void* stream);
int althea_ibl_batch_describe(const althea_ibl_batch* batch, althea_ibl_batch_info* info);
/* Synchronises `stream` and reports the last run: ALTHEA_IBL_ERR_CUDA when a
 * bounded wait of the precision path's contraction gave up (the outputs of
 * that run are then undefined), else ALTHEA_IBL_OK. */
int althea_ibl_batch_status(const althea_ibl_batch* batch, void* stream);
int althea_ibl_batch_destroy(althea_ibl_batch* batch);

/* ---- analytic sun lobes ---------------------------------------------------------
 * No counterpart in the reference, whose env maps are fixed files
 * (Src/ImageBasedLighting.cpp:429-446).  A probe is usually re-baked because
 * its lights changed (the sun moved with the time of day), not its whole sky:
 * these calls add Gaussian sun lobes to a sky map on the device,
 *   out = base + sum_s radiance_s exp(-theta_s^2 / (2 sigma_s^2))  on R, G, B,
 * theta_s = angle between a texel centre's direction and dir_s, with the
 * texel directions of sampleEnvMap (PreFilterEnvMap.comp:98-122); alpha is
 * copied.  The server applies a request's suns to a resident map before its
 * bake.  out_dev may equal base_dev (RGBA32F, width x height, tightly packed). */
#define ALTHEA_IBL_MAX_SUNS 16
typedef struct {
  float dir[3];              /* direction (x, y, z); normalised by the call */
  float sigma;               /* angular width in radians, 0 < sigma < 4 */
  float radiance;            /* peak radiance added to R, G and B, >= 0 */
} althea_ibl_sun;
int althea_ibl_apply_suns(const float* base_dev, float* out_dev, int width, int height,
                          const althea_ibl_sun* suns, int sun_count, void* stream);

/* ---- serving: continuous re-bakes under an HBM budget -------------------------
 * No counterpart in the reference (one synchronous bake at start-up,
 * Src/GlobalResources.cpp:18-22).  A server admits probe re-bake requests as
 * they arrive: a request starts as soon as a slot (a CUDA stream) is free and
 * its device memory (env chain, outputs, scratch) fits the budget; requests
 * that do not fit wait in FIFO order.  Admitted requests run concurrently on
 * their own streams; buffers are recycled through a size-class pool (no
 * cudaFree on the request path).  Results are identical whether a request runs
 * alone or among others (the kernels are deterministic and independent of
 * concurrency).  The API is single-threaded: call submit/poll from one thread. */
typedef struct {
  size_t budget_bytes;       /* device memory the server may hold */
  int max_inflight;          /* requests on the GPU at once (streams) */
  int samples, generator;    /* prefilter sample count and generator (plain path) */
  int irradiance_width, irradiance_height;
  int path;                  /* ALTHEA_IBL_PATH_*; the precision workspace counts against
                                the budget */
} althea_ibl_server_config;

typedef struct {
  const float* env_host;     /* RGBA32F level 0, host memory (pinned for overlap);
                                unused (may be NULL) when env_id names a resident map */
  int env_width, env_height; /* with env_id: the registered map's size */
  int mip_count;             /* mips from W/2 x H/2, roughness m/(M-1) */
  float* irradiance_host;    /* irradiance_width*height*4 floats, or NULL */
  float* mips_host;          /* every mip back to back (sum of w*h*4 floats) */
  uint64_t tag;
  int env_id;                /* 0: upload env_host; else an id from
                                althea_ibl_server_register_env (the map stays on the device) */
  int sun_count;             /* suns added to the map before the bake, 0..ALTHEA_IBL_MAX_SUNS */
  althea_ibl_sun suns[ALTHEA_IBL_MAX_SUNS];
} althea_ibl_request;

typedef struct {
  uint64_t tag;
  int status;                /* althea_ibl_status of the request */
  double submit_s, start_s, done_s;   /* steady-clock seconds */
} althea_ibl_completion;

typedef struct {
  int inflight, queued;
  size_t bytes_in_use, bytes_reserved, peak_bytes_in_use;
  uint64_t completed, rejected;
  size_t bytes_resident;     /* registered env maps */
  int resident_maps;
} althea_ibl_server_stats;

typedef struct althea_ibl_server althea_ibl_server;

int althea_ibl_server_create(const althea_ibl_server_config* cfg, althea_ibl_server** out);
/* Queues the request and admits what fits; never blocks on the GPU.  A request
 * whose memory alone exceeds the budget is refused with ALTHEA_IBL_ERR_BUDGET;
 * on the precision path, a shape the planner cannot run is refused with
 * ALTHEA_IBL_ERR_UNSUPPORTED. */
int althea_ibl_server_submit(althea_ibl_server* s, const althea_ibl_request* req);
/* Retires finished requests (returning up to max completions), frees their
 * slots and memory, and admits queued requests that now fit. */
int althea_ibl_server_poll(althea_ibl_server* s, althea_ibl_completion* out, int max, int* n);
int althea_ibl_server_get_stats(const althea_ibl_server* s, althea_ibl_server_stats* st);
/* Resident env maps.  register uploads an RGBA32F level 0 (host memory, or
 * device memory when src_is_device) once and keeps it on the device, counted
 * against the budget, until unregister; requests then name it by env_id and
 * move no env map across the host link (a re-bake of a known sky, with the
 * request's suns added on the device).  register refuses a map that does not
 * fit the budget beside what the server already holds (ALTHEA_IBL_ERR_BUDGET);
 * unregister refuses while queued or running requests use the map
 * (ALTHEA_IBL_ERR_NOT_READY).  Synchronous (not on the request path). */
int althea_ibl_server_register_env(althea_ibl_server* s, const float* rgba, int env_width,
                                   int env_height, int src_is_device, int* env_id_out);
int althea_ibl_server_unregister_env(althea_ibl_server* s, int env_id);
/* Device memory a request of this size holds while in flight; 0 for a size
 * the server cannot run. */
size_t althea_ibl_server_request_bytes(const althea_ibl_server* s, int env_width, int env_height,
                                       int mip_count);
double althea_ibl_server_now(void);   /* the steady clock used in completions */
/* Waits for everything in flight, then releases all device memory. */
int althea_ibl_server_destroy(althea_ibl_server* s);

/* ---- Radiance .hdr (RGBE) files: the bake cache format ---------------------
 * Replaces Utilities::loadHdri / saveHdri (Src/Utilities.cpp:216-255, stb) as
 * used by the bake cache (Src/ImageBasedLighting.cpp:58-102,429-446,483-568).
 * Host memory, RGBA32F with alpha 1, row 0 = first scanline.  read allocates
 * *rgba_out (free it with althea_ibl_hdr_free); write run-length encodes
 * scanlines 8..32767 wide. */
int althea_ibl_hdr_read(const char* path, float** rgba_out, int* width, int* height);
void althea_ibl_hdr_free(float* rgba);
int althea_ibl_hdr_write(const char* path, const float* rgba, int width, int height);

/* ---- Reflection-buffer glossy convolution ----------------------------------
 * Replaces ReflectionBuffer::convolveReflectionBuffer (Src/ReflectionBuffer.cpp:
 * 163-275), the per-frame dispatch of Shaders/SSRGlossyConvolve.comp:25-53 over
 * the RGBA16F reflection buffer (Src/ReflectionBuffer.cpp:28-36): levels
 * 1..mip_count-1 become the 7-tap Gaussian of the level before, vertical for odd
 * levels and horizontal for even ones, bit-identical to the shader's FP32
 * arithmetic with a Vulkan LINEAR / CLAMP_TO_EDGE sampler.  Level l is
 * max(1, width >> l) x max(1, height >> l) texels of 4 IEEE halfs (8 bytes);
 * mip_count 1..16 (the reference uses 5).  Launches only; no allocation.
 *
 * althea_ssr_convolve: every level packed back to back in one device buffer,
 *   level l at texel althea_ssr_level_offset(width, height, l).
 * althea_ssr_convolve_levels: one device pointer and row pitch (bytes, a
 *   multiple of 8) per level, e.g. buffers imported per mip. */
size_t althea_ssr_level_offset(int width, int height, int level);  /* in texels */
int althea_ssr_convolve(void* chain_dev, int width, int height, int mip_count, void* stream);
int althea_ssr_convolve_levels(void* const* levels_dev, const size_t* pitch_bytes, int width,
                               int height, int mip_count, void* stream);

const char* althea_ibl_last_error(void);
int althea_ibl_abi_version(void);

#ifdef __cplusplus
}
#endif
#endif /* ALTHEA_IBL_H */
