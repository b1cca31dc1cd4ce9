// ibl_plain.cu -- plain (reference-estimator) IBL kernels for sm_103a and the
// stateless C-ABI entry points of include/althea_ibl.h.
//
// Compiled with -fmad=false (see ibl_device.cuh): outputs equal the CPU
// restatement of the reference shaders bit for bit, except the irradiance sum,
// which is split across threads (tree order instead of serial order; ~1e-7).
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdio>
#include <cstring>

#include "althea_ibl.h"
#include "ibl_internal.h"
#include "ibl_texel.cuh"

namespace ibl {

// ---------------------------------------------------------------------------
// Error reporting shared by every entry point.
// ---------------------------------------------------------------------------
static thread_local char g_last_error[512] = "";

int set_error(int status, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
  va_end(ap);
  return status;
}

int cuda_status(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return ALTHEA_IBL_OK;
  int st = e == cudaErrorMemoryAllocation ? ALTHEA_IBL_ERR_OUT_OF_MEMORY : ALTHEA_IBL_ERR_CUDA;
  return set_error(st, "%s: %s", what, cudaGetErrorString(e));
}

const char* last_error() { return g_last_error; }

// ---------------------------------------------------------------------------
// Mip chain: vkCmdBlitImage(VK_FILTER_LINEAR) per level (Src/Image.cpp:184-213).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) blit_level_kernel(const float4* __restrict__ src, int sw,
                                                         int sh, float4* __restrict__ dst, int dw,
                                                         int dh) {
  int x = blockIdx.x * 32 + (threadIdx.x & 31);
  int y = blockIdx.y * 8 + (threadIdx.x >> 5);
  if (x >= dw || y >= dh) return;
  dst[(long long)y * dw + x] = blit_texel(src, sw, sh, dw, dh, x, y);
}

int launch_build_chain(const float* level0, int w, int h, float* chain, cudaStream_t st) {
  ChainTable t;
  make_table(w, h, &t);
  float4* c = reinterpret_cast<float4*>(chain);
  if (level0 != chain) {
    cudaError_t e = cudaMemcpyAsync(c, level0, (size_t)w * h * sizeof(float4),
                                    cudaMemcpyDeviceToDevice, st);
    if (e != cudaSuccess) return cuda_status(e, "level-0 copy");
  }
  for (int l = 1; l < t.levels; ++l) {
    dim3 grid((t.lw[l] + 31) / 32, (t.lh[l] + 7) / 8);
    blit_level_kernel<<<grid, 256, 0, st>>>(c + t.off[l - 1], t.lw[l - 1], t.lh[l - 1],
                                            c + t.off[l], t.lw[l], t.lh[l]);
  }
  return cuda_status(cudaGetLastError(), "blit_level_kernel launch");
}

// ---------------------------------------------------------------------------
// GGX prefilter (PreFilterEnvMap.comp:126-177).  One thread = one output
// texel, samples accumulated serially in the shader's order; every mip of
// the chain in one launch (block ranges per mip).
// ---------------------------------------------------------------------------
constexpr int kPfTileX = 16, kPfTileY = 8;

struct PrefilterJob {
  float4* out;
  long long pitch;  // in texels
  int ow, oh;
  float roughness;
  int tiles_x;
  int block_begin;
};

struct PrefilterParams {
  const float4* chain;
  int w, h;
  int samples;
  int generator;
  int njobs;
  int tabulate;  // Hammersley and samples <= kMaxTabulatedSamples
  PrefilterJob jobs[ALTHEA_IBL_MAX_MIPS];
};

__global__ void __launch_bounds__(kPfTileX* kPfTileY) prefilter_kernel(const PrefilterParams p) {
  __shared__ ChainTable tab;
  __shared__ PrefilterJob job;
  extern __shared__ float h_local[];  // 3 * samples floats when tabulated
  if (threadIdx.x == 0) {
    make_table(p.w, p.h, &tab);
    int sel = 0;
#pragma unroll
    for (int k = 1; k < ALTHEA_IBL_MAX_MIPS; ++k)
      if (k < p.njobs && (int)blockIdx.x >= p.jobs[k].block_begin) sel = k;
#pragma unroll
    for (int k = 0; k < ALTHEA_IBL_MAX_MIPS; ++k)
      if (k == sel) job = p.jobs[k];
  }
  __syncthreads();
  const bool tabulated = p.tabulate && job.roughness != 0.0f;
  if (tabulated) {
    tabulate_hammersley(h_local, p.samples, job.roughness);
    __syncthreads();
  }
  int local = (int)blockIdx.x - job.block_begin;
  int x = (local % job.tiles_x) * kPfTileX + (int)(threadIdx.x % kPfTileX);
  int y = (local / job.tiles_x) * kPfTileY + (int)(threadIdx.x / kPfTileX);
  if (x >= job.ow || y >= job.oh) return;
  job.out[(long long)y * job.pitch + x] =
      prefilter_texel(p.chain, tab, p.w, p.h, x, y, job.ow, job.oh, job.roughness, p.samples,
                      p.generator, tabulated ? h_local : nullptr);
}

// The value a delta lobe (roughness 0) converges to: the one reflected sample
// that every kept sample of PreFilterEnvMap.comp:147-167 repeats (H = N, first
// Hammersley point), without repeating its accumulation.  The precision path
// uses it for roughness-0 mips (its quadrature of a delta).
// Texel (x, y) of a delta mip (the caller's 32 x 8 block of 256 threads).
__device__ __forceinline__ void delta_texel(const float4* __restrict__ chain,
                                            const ChainTable& tab, void* __restrict__ out,
                                            long long pitch, int ow, int oh, int out_half, int x,
                                            int y) {
  if (x >= ow || y >= oh) return;
  Float3 n = texel_dir(x, y, ow, oh);
  Float3 t, b;
  local_frame(n, t, b);
  Float3 hv = to_world(t, b, n, sample_ggx(0.0f, 0.0f, 0.0f));
  float vdh = (n.x * hv.x + n.y * hv.y) + n.z * hv.z;
  float k = 2.0f * vdh;
  Float3 l = normalize3(f3(k * hv.x - n.x, k * hv.y - n.y, k * hv.z - n.z));
  float ndotl = glsl_max((n.x * l.x + n.y * l.y) + n.z * l.z, 0.0f);
  float4 o = make_float4(0.0f, 0.0f, 0.0f, 1.0f);
  if (ndotl > 0.0f) {
    Float3 c = sample_env(chain, tab, l, 0.0f);
    o = make_float4(c.x, c.y, c.z, 1.0f);
  }
  if (out_half) {
    const __half2 rg = __floats2half2_rn(o.x, o.y), ba = __floats2half2_rn(o.z, o.w);
    uint2 v;
    v.x = *reinterpret_cast<const uint32_t*>(&rg);
    v.y = *reinterpret_cast<const uint32_t*>(&ba);
    reinterpret_cast<uint2*>(out)[(long long)y * pitch + x] = v;
  } else {
    reinterpret_cast<float4*>(out)[(long long)y * pitch + x] = o;
  }
}

__global__ void __launch_bounds__(256) delta_mip_kernel(const float4* __restrict__ chain, int w,
                                                        int h, void* __restrict__ out,
                                                        long long pitch, int ow, int oh,
                                                        int out_half) {
  __shared__ ChainTable tab;
  if (threadIdx.x == 0) make_table(w, h, &tab);
  __syncthreads();
  delta_texel(chain, tab, out, pitch, ow, oh, out_half,
              blockIdx.x * 32 + (int)(threadIdx.x & 31), blockIdx.y * 8 + (int)(threadIdx.x >> 5));
}

// The delta mips of many probes in one launch: block b is block b - begins[k]
// of job k's (ceil(ow / 32) x ceil(oh / 8)) grid, row-major.
__global__ void __launch_bounds__(256) delta_batch_kernel(const DeltaJob* __restrict__ jobs,
                                                          const long long* __restrict__ begins,
                                                          int njobs) {
  __shared__ ChainTable tab;
  __shared__ int k_sh;
  if (threadIdx.x == 0) {
    k_sh = find_range(begins, njobs, blockIdx.x);
    make_table(jobs[k_sh].w, jobs[k_sh].h, &tab);
  }
  __syncthreads();
  const DeltaJob& j = jobs[k_sh];
  const long long local = (long long)blockIdx.x - begins[k_sh];
  const int bx = (int)(local % j.blocks_x), by = (int)(local / j.blocks_x);
  delta_texel(reinterpret_cast<const float4*>(j.chain), tab, j.out, j.pitch, j.ow, j.oh,
              j.out_half, bx * 32 + (int)(threadIdx.x & 31), by * 8 + (int)(threadIdx.x >> 5));
}

int launch_delta_mip(const float* chain, int w, int h, const althea_ibl_mip_target* mip,
                     int out_half, cudaStream_t st) {
  dim3 grid((mip->width + 31) / 32, (mip->height + 7) / 8);
  delta_mip_kernel<<<grid, 256, 0, st>>>(reinterpret_cast<const float4*>(chain), w, h,
                                         mip->out_dev,
                                         (long long)(mip->pitch_bytes / (out_half ? 8 : 16)),
                                         mip->width, mip->height, out_half);
  return cuda_status(cudaGetLastError(), "delta mip launch");
}

int launch_delta_batch(const DeltaJob* d_jobs, const long long* d_begins, int njobs,
                       long long blocks, cudaStream_t st) {
  if (njobs <= 0 || blocks <= 0) return ALTHEA_IBL_OK;
  delta_batch_kernel<<<(unsigned)blocks, 256, 0, st>>>(d_jobs, d_begins, njobs);
  return cuda_status(cudaGetLastError(), "delta batch launch");
}

int launch_prefilter(const float* chain, int w, int h, const althea_ibl_mip_target* mips,
                     int mip_count, int samples, int generator, cudaStream_t st) {
  PrefilterParams p;
  memset(&p, 0, sizeof(p));
  p.chain = reinterpret_cast<const float4*>(chain);
  p.w = w;
  p.h = h;
  p.samples = samples;
  p.generator = generator;
  p.njobs = mip_count;
  int blocks = 0;
  for (int m = 0; m < mip_count; ++m) {
    PrefilterJob& j = p.jobs[m];
    j.out = reinterpret_cast<float4*>(mips[m].out_dev);
    j.pitch = (long long)(mips[m].pitch_bytes / sizeof(float4));
    j.ow = mips[m].width;
    j.oh = mips[m].height;
    j.roughness = mips[m].roughness;
    j.tiles_x = (j.ow + kPfTileX - 1) / kPfTileX;
    j.block_begin = blocks;
    blocks += j.tiles_x * ((j.oh + kPfTileY - 1) / kPfTileY);
  }
  if (blocks == 0) return ALTHEA_IBL_OK;
  p.tabulate = generator == ALTHEA_IBL_GEN_HAMMERSLEY && samples <= kMaxTabulatedSamples;
  size_t smem = p.tabulate ? 3 * (size_t)samples * sizeof(float) : 0;
  prefilter_kernel<<<blocks, kPfTileX * kPfTileY, smem, st>>>(p);
  return cuda_status(cudaGetLastError(), "prefilter_kernel launch");
}

// ---------------------------------------------------------------------------
// Irradiance (GenIrradianceMap.comp:106-155).  One output texel's 300 x Nphi
// grid is cut into 32 fixed bands of theta rows, summed by warps whose 32
// lanes cover a 4 (theta) x 8 (phi) patch of neighbouring grid directions
// (so one gather instruction touches a compact patch of the env level); band
// sums are combined by one fixed binary tree.  GB = 1, 2 or 4 blocks share a
// texel, each reducing an aligned subtree; a second kernel applies the top
// levels.  Deterministic, independent of GB, and within float rounding of the
// shader's serial sum.
// ---------------------------------------------------------------------------
IrrPlan irr_plan(int w, int h, int ow, int oh, int target_blocks) {
  IrrPlan pl;
  pl.phi = irr_phi_samples(w, h);
  long long texels = (long long)ow * oh;
  pl.texels = texels;
  if (target_blocks <= 0) target_blocks = 152 * 8;
  pl.gb = irradiance_split(texels, target_blocks);
  pl.workspace = (size_t)texels * (size_t)pl.gb * sizeof(float4);
  return pl;
}

__global__ void __launch_bounds__(32 * kIrrWarps) irradiance_partial_kernel(
    const float4* __restrict__ chain, int w, int h, int ow, int oh, int gb_count, int phi_samples,
    float4* __restrict__ partial) {
  __shared__ ChainTable tab;
  __shared__ float cos_t[kThetaSamples], sin_t[kThetaSamples];
  __shared__ float band_smem[kBands][3];
  extern __shared__ float phi_table[];  // 2 * phi_samples floats
  float* cos_p = phi_table;
  float* sin_p = phi_table + phi_samples;
  if (threadIdx.x == 0) make_table(w, h, &tab);
  irradiance_tables(cos_t, sin_t, cos_p, sin_p, phi_samples);
  __syncthreads();

  const long long texel = blockIdx.x / gb_count;
  const int gb = blockIdx.x % gb_count;
  const int count = kBands / gb_count;
  Float3 s = irradiance_block_bands(chain, tab, w, (int)(texel % ow), (int)(texel / ow), ow, oh,
                                    gb * count, count, phi_samples, cos_t, sin_t, cos_p, sin_p,
                                    band_smem);
  if (threadIdx.x == 0) partial[texel * gb_count + gb] = make_float4(s.x, s.y, s.z, 0.0f);
}

__global__ void __launch_bounds__(256) irradiance_finish_kernel(const float4* __restrict__ partial,
                                                                int ow, int oh, int gb_count,
                                                                int phi_samples,
                                                                float4* __restrict__ out,
                                                                long long pitch) {
  long long texel = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (texel >= (long long)ow * oh) return;
  int x = (int)(texel % ow), y = (int)(texel / ow);
  Float3 s = combine_partials(partial + texel * gb_count, gb_count);
  out[(long long)y * pitch + x] = irradiance_finish(s.x, s.y, s.z, phi_samples);
}

int launch_irradiance(const float* chain, int w, int h, float* out, int ow, int oh,
                      size_t pitch_bytes, void* ws, cudaStream_t st) {
  IrrPlan pl = irr_plan(w, h, ow, oh);
  float4* partial = reinterpret_cast<float4*>(ws);
  long long blocks = pl.texels * pl.gb;
  if (blocks > 0x7fffffffLL)
    return set_error(ALTHEA_IBL_ERR_UNSUPPORTED, "irradiance output too large");
  size_t smem = 2 * (size_t)pl.phi * sizeof(float);
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(irradiance_partial_kernel,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return cuda_status(e, "irradiance smem attribute");
  }
  irradiance_partial_kernel<<<(unsigned)blocks, 32 * kIrrWarps, smem, st>>>(
      reinterpret_cast<const float4*>(chain), w, h, ow, oh, pl.gb, pl.phi, partial);
  long long n = pl.texels;
  irradiance_finish_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(
      partial, ow, oh, pl.gb, pl.phi, reinterpret_cast<float4*>(out),
      (long long)(pitch_bytes / sizeof(float4)));
  return cuda_status(cudaGetLastError(), "irradiance kernels launch");
}
// ---------------------------------------------------------------------------
// Split-sum BRDF LUT (Karis 2013, IntegrateBRDF).  One thread per texel, N
// Hammersley samples in order; FP32 (it is not a contraction).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) brdf_lut_kernel(float2* __restrict__ out, int n,
                                                       long long pitch, int samples,
                                                       int orientation) {
  int i = blockIdx.x * 32 + (threadIdx.x & 31);
  int j = blockIdx.y * 8 + (threadIdx.x >> 5);
  if (i >= n || j >= n) return;
  float nov = ((float)i + 0.5f) / (float)n;
  float tj = ((float)j + 0.5f) / (float)n;
  float rough = orientation == ALTHEA_IBL_LUT_ASSET ? 1.0f - tj : tj;
  float vx = sqrtf(1.0f - nov * nov), vz = nov;
  float alpha = rough * rough;
  float a2 = alpha * alpha;
  float k = alpha / 2.0f;
  // G1(V) / NoV once per texel, 1 / NoH once per sample
  const float gv = 1.0f / (nov * (1.0f - k) + k);
  float sum_a = 0.0f, sum_b = 0.0f;
#pragma unroll 1
  for (int s = 0; s < samples; ++s) {
    float xi_x, xi_y;
    hammersley(s, samples, xi_x, xi_y);
    float phi = 2.0f * kPi * xi_x;
    float cos_t = sqrtf((1.0f - xi_y) / (1.0f + (a2 - 1.0f) * xi_y));
    float sin_t = sqrtf(1.0f - cos_t * cos_t);
    float hx = sin_t * agb_cos(phi), hz = cos_t;
    float noh = hz > 0.0f ? (hz < 1.0f ? hz : 1.0f) : 0.0f;
    agb_lut_sample(vx, vz, hx, hz, 1.0f / noh, 1.0f - k, k, gv, &sum_a, &sum_b);
  }
  out[(long long)j * pitch + i] = make_float2(sum_a / (float)samples, sum_b / (float)samples);
}

// The same estimator with the half-vector samples of a row (they depend on the
// roughness only, not on N.V) tabulated once in shared memory: every texel
// evaluates the identical IEEE operations in the identical order, so the
// result is bit-identical to brdf_lut_kernel.  Block per (row, 256 columns);
// dynamic shared memory: samples * 16 bytes.
constexpr int kLutTableMax = 8192;

__global__ void __launch_bounds__(256) brdf_lut_row_kernel(float2* __restrict__ out, int n,
                                                           long long pitch, int samples,
                                                           int orientation) {
  extern __shared__ float4 hsamp[];  // (hx, hz, 1 / NoH, -) per sample
  const int j = blockIdx.y;
  float tj = ((float)j + 0.5f) / (float)n;
  float rough = orientation == ALTHEA_IBL_LUT_ASSET ? 1.0f - tj : tj;
  float alpha = rough * rough;
  float a2 = alpha * alpha;
  float k = alpha / 2.0f;
  for (int s = threadIdx.x; s < samples; s += blockDim.x) {
    float xi_x, xi_y;
    hammersley(s, samples, xi_x, xi_y);
    float phi = 2.0f * kPi * xi_x;
    float cos_t = sqrtf((1.0f - xi_y) / (1.0f + (a2 - 1.0f) * xi_y));
    float sin_t = sqrtf(1.0f - cos_t * cos_t);
    const float hz = cos_t, noh = hz > 0.0f ? (hz < 1.0f ? hz : 1.0f) : 0.0f;
    hsamp[s] = make_float4(sin_t * agb_cos(phi), cos_t, 1.0f / noh, 0.0f);
  }
  __syncthreads();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float nov = ((float)i + 0.5f) / (float)n;
  float vx = sqrtf(1.0f - nov * nov), vz = nov;
  // G1(V) / NoV once per texel; 1 / NoH comes with the sample
  const float gv = 1.0f / (nov * (1.0f - k) + k);
  float sum_a = 0.0f, sum_b = 0.0f;
  const float omk = 1.0f - k;
#pragma unroll 4
  for (int s = 0; s < samples; ++s) {
    const float4 hv = hsamp[s];
    agb_lut_sample(vx, vz, hv.x, hv.y, hv.z, omk, k, gv, &sum_a, &sum_b);
  }
  out[(long long)j * pitch + i] = make_float2(sum_a / (float)samples, sum_b / (float)samples);
}

int launch_brdf_lut(float* out, int n, size_t pitch_bytes, int samples, int orientation,
                    cudaStream_t st) {
  const long long pitch = (long long)(pitch_bytes / sizeof(float2));
  if (samples <= kLutTableMax) {
    const int sm = samples * (int)sizeof(float4);
    if (sm > 48 * 1024) {
      cudaError_t e = cudaFuncSetAttribute(brdf_lut_row_kernel,
                                           cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
      if (e != cudaSuccess) return cuda_status(e, "brdf lut smem attribute");
    }
    dim3 grid((n + 255) / 256, n);
    brdf_lut_row_kernel<<<grid, 256, sm, st>>>(reinterpret_cast<float2*>(out), n, pitch, samples,
                                               orientation);
  } else {
    dim3 grid((n + 31) / 32, (n + 7) / 8);
    brdf_lut_kernel<<<grid, 256, 0, st>>>(reinterpret_cast<float2*>(out), n, pitch, samples,
                                          orientation);
  }
  return cuda_status(cudaGetLastError(), "brdf lut launch");
}

// ---------------------------------------------------------------------------
// Argument checks shared with the context API.
// ---------------------------------------------------------------------------
int check_env(int w, int h) {
  if (w < 1 || h < 1 || w > 32768 || h > 32768)
    return set_error(ALTHEA_IBL_ERR_INVALID_ARGUMENT,
                     "env size %dx%d outside 1..32768 per side", w, h);
  return ALTHEA_IBL_OK;
}

int check_image(const void* p, int w, int h, size_t pitch, size_t texel_bytes, const char* what) {
  if (!p) return set_error(ALTHEA_IBL_ERR_INVALID_ARGUMENT, "%s: null pointer", what);
  if (w < 1 || h < 1 || w > 65536 || h > 65536)
    return set_error(ALTHEA_IBL_ERR_INVALID_ARGUMENT, "%s: bad size %dx%d", what, w, h);
  if (pitch < (size_t)w * texel_bytes || pitch % texel_bytes != 0)
    return set_error(ALTHEA_IBL_ERR_INVALID_ARGUMENT,
                     "%s: pitch %zu bytes must be a multiple of %zu and >= %zu", what, pitch,
                     texel_bytes, (size_t)w * texel_bytes);
  if (((uintptr_t)p) % texel_bytes != 0)
    return set_error(ALTHEA_IBL_ERR_INVALID_ARGUMENT, "%s: pointer not %zu-byte aligned", what,
                     texel_bytes);
  return ALTHEA_IBL_OK;
}

int check_irradiance_args(int w, int h, int ow, int oh) {
  int phi = irr_phi_samples(w, h);
  if (phi < 1 || phi > kMaxPhiSamples)
    return set_error(ALTHEA_IBL_ERR_UNSUPPORTED,
                     "irradiance grid int(300*H/W) = %d for %dx%d; supported 1..%d", phi, w, h,
                     kMaxPhiSamples);
  if (ow < 1 || oh < 1 || ow > 65536 || oh > 65536)
    return set_error(ALTHEA_IBL_ERR_INVALID_ARGUMENT, "irradiance size %dx%d outside 1..65536",
                     ow, oh);
  return ALTHEA_IBL_OK;
}

}  // namespace ibl

// ===========================================================================
// Stateless C ABI.
// ===========================================================================
using namespace ibl;

extern "C" int althea_ibl_abi_version(void) { return ALTHEA_IBL_ABI_VERSION; }

extern "C" const char* althea_ibl_last_error(void) { return ibl::last_error(); }

extern "C" int althea_ibl_chain_levels(int w, int h) {
  if (check_env(w, h) != ALTHEA_IBL_OK) return 0;
  return chain_levels(w, h);
}

extern "C" size_t althea_ibl_chain_texels(int w, int h) {
  if (check_env(w, h) != ALTHEA_IBL_OK) return 0;
  ChainTable t;
  make_table(w, h, &t);
  return (size_t)(t.off[t.levels - 1] + (long long)t.lw[t.levels - 1] * t.lh[t.levels - 1]);
}

extern "C" size_t althea_ibl_chain_level_offset(int w, int h, int level) {
  if (check_env(w, h) != ALTHEA_IBL_OK) return 0;
  ChainTable t;
  make_table(w, h, &t);
  if (level < 0 || level >= t.levels) return 0;
  return (size_t)t.off[level];
}

extern "C" int althea_ibl_build_env_chain(const float* level0, int w, int h, float* chain,
                                          void* stream) {
  int st = check_env(w, h);
  if (st) return st;
  if (!level0 || !chain) return set_error(ALTHEA_IBL_ERR_INVALID_ARGUMENT, "null pointer");
  if (((uintptr_t)level0 | (uintptr_t)chain) % 16)
    return set_error(ALTHEA_IBL_ERR_INVALID_ARGUMENT, "chain pointers must be 16-byte aligned");
  return launch_build_chain(level0, w, h, chain, (cudaStream_t)stream);
}

extern "C" int althea_ibl_prefilter(const float* chain, int w, int h,
                                    const althea_ibl_mip_target* mips, int mip_count,
                                    int samples, int generator, void* stream) {
  ibl::NvtxRange nvtx_range("althea_ibl_prefilter");
  int st = check_env(w, h);
  if (st) return st;
  if (!chain || ((uintptr_t)chain) % 16)
    return set_error(ALTHEA_IBL_ERR_INVALID_ARGUMENT, "chain: null or not 16-byte aligned");
  if (mip_count < 0 || mip_count > ALTHEA_IBL_MAX_MIPS || (mip_count > 0 && !mips))
    return set_error(ALTHEA_IBL_ERR_INVALID_ARGUMENT, "mip_count %d outside 0..%d", mip_count,
                     ALTHEA_IBL_MAX_MIPS);
  if (samples < 1 || samples > (1 << 24))
    return set_error(ALTHEA_IBL_ERR_INVALID_ARGUMENT, "samples %d outside 1..2^24", samples);
  if (generator != ALTHEA_IBL_GEN_REF_HASH && generator != ALTHEA_IBL_GEN_HAMMERSLEY)
    return set_error(ALTHEA_IBL_ERR_INVALID_ARGUMENT, "unknown generator %d", generator);
  for (int m = 0; m < mip_count; ++m) {
    st = check_image(mips[m].out_dev, mips[m].width, mips[m].height, mips[m].pitch_bytes, 16,
                     "prefilter mip");
    if (st) return st;
    float r = mips[m].roughness;
    if (!(r >= 0.0f && r <= 1.0f))
      return set_error(ALTHEA_IBL_ERR_INVALID_ARGUMENT, "mip %d roughness %g outside [0,1]", m,
                       (double)r);
  }
  return launch_prefilter(chain, w, h, mips, mip_count, samples, generator,
                          (cudaStream_t)stream);
}

extern "C" size_t althea_ibl_irradiance_workspace_size(int w, int h, int ow, int oh) {
  if (check_env(w, h) || check_irradiance_args(w, h, ow, oh)) return 0;
  return irr_plan(w, h, ow, oh).workspace;
}

extern "C" int althea_ibl_irradiance(const float* chain, int w, int h, float* out, int ow, int oh,
                                     size_t pitch, void* ws, size_t ws_bytes, void* stream) {
  ibl::NvtxRange nvtx_range("althea_ibl_irradiance");
  int st = check_env(w, h);
  if (st) return st;
  st = check_irradiance_args(w, h, ow, oh);
  if (st) return st;
  if (!chain || ((uintptr_t)chain) % 16)
    return set_error(ALTHEA_IBL_ERR_INVALID_ARGUMENT, "chain: null or not 16-byte aligned");
  st = check_image(out, ow, oh, pitch, 16, "irradiance");
  if (st) return st;
  IrrPlan pl = irr_plan(w, h, ow, oh);
  if (!ws || ws_bytes < pl.workspace || ((uintptr_t)ws) % 16)
    return set_error(ALTHEA_IBL_ERR_INVALID_ARGUMENT,
                     "irradiance workspace needs %zu bytes (16-byte aligned), got %zu",
                     pl.workspace, ws_bytes);
  return launch_irradiance(chain, w, h, out, ow, oh, pitch, ws, (cudaStream_t)stream);
}

extern "C" int althea_ibl_brdf_lut(float* out, int n, size_t pitch, int samples, int orientation,
                                   void* stream) {
  if (n < 1 || n > 16384) return set_error(ALTHEA_IBL_ERR_INVALID_ARGUMENT, "LUT size %d", n);
  int st = check_image(out, n, n, pitch, 8, "brdf lut");
  if (st) return st;
  if (samples < 1 || samples > (1 << 24))
    return set_error(ALTHEA_IBL_ERR_INVALID_ARGUMENT, "LUT samples %d", samples);
  if (orientation != ALTHEA_IBL_LUT_ASSET && orientation != ALTHEA_IBL_LUT_CORRECTED)
    return set_error(ALTHEA_IBL_ERR_INVALID_ARGUMENT, "LUT orientation %d", orientation);
  return launch_brdf_lut(out, n, pitch, samples, orientation, (cudaStream_t)stream);
}
