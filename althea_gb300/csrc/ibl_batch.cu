// ibl_batch.cu -- many probes of uneven size in one CUDA-graph launch.
//
// A plan (althea_ibl_batch_create) turns a probe table into device job tables:
//  * chain jobs per level index (one launch per level over every probe that
//    has the level; level 0 is a copy from the caller's level-0 buffer);
//  * a (probe, mip, tile) work queue drained by a persistent prefilter kernel
//    through one atomic counter -- full-sample jobs first, the cheap
//    roughness-0 jobs last, so the tail of the queue is short;
//  * (probe, texel, split) blocks of a batched irradiance plus its finish;
//  * an optional shared BRDF LUT.
// Every texel runs the same per-texel code as the single-probe kernels
// (ibl_texel.cuh), so a batch equals baking each probe alone, bit for bit.
// The whole bake is captured once into a CUDA graph and replayed.
//
// Autotuner: candidate prefilter tile shapes and irradiance split targets are
// timed with CUDA events on the first plan of a given batch shape; the
// winner is cached per shape key in memory and, when $ALTHEA_IBL_TUNE_CACHE
// names a file, on disk (one "key tile_x tile_y irr_target" line per shape).
//
// Compiled with -fmad=false (bit parity with the oracle).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <new>
#include <sstream>
#include <string>
#include <vector>

#include "althea_ibl.h"
#include "ibl_internal.h"
#include "ibl_texel.cuh"

namespace ibl {
namespace {

struct BlitJob {
  const float4* src;
  float4* dst;
  int sw, sh, dw, dh;
  int blocks_x;
  int copy;  // level 0: plain copy from the caller's buffer
};

struct PfJob {
  const float4* chain;
  float4* out;
  long long pitch;
  int w, h, ow, oh;
  float roughness;
  int tiles_x;
};

struct IrrJob {
  const float4* chain;
  float4* out;
  long long pitch;
  int w, h, ow, oh, gb, phi;
  long long partial_offset;
};

__global__ void __launch_bounds__(256) batch_blit_kernel(const BlitJob* __restrict__ jobs,
                                                         const long long* __restrict__ begins,
                                                         int njobs) {
  __shared__ int s_job;
  if (threadIdx.x == 0) s_job = find_range(begins, njobs, blockIdx.x);
  __syncthreads();
  const BlitJob j = jobs[s_job];
  long long local = (long long)blockIdx.x - begins[s_job];
  int x = (int)(local % j.blocks_x) * 32 + (threadIdx.x & 31);
  int y = (int)(local / j.blocks_x) * 8 + (threadIdx.x >> 5);
  if (x >= j.dw || y >= j.dh) return;
  long long o = (long long)y * j.dw + x;
  j.dst[o] = j.copy ? __ldg(j.src + o) : blit_texel(j.src, j.sw, j.sh, j.dw, j.dh, x, y);
}

template <int TX, int TY>
__global__ void __launch_bounds__(TX* TY) batch_prefilter_kernel(
    const PfJob* __restrict__ jobs, const long long* __restrict__ begins, int njobs,
    long long total_tiles, int samples, int generator, int tabulate,
    unsigned long long* __restrict__ counter) {
  __shared__ ChainTable tab;
  __shared__ PfJob job;
  __shared__ long long s_tile;
  __shared__ int s_job;
  __shared__ float s_tab_rough;
  extern __shared__ float h_local[];
  if (threadIdx.x == 0) {
    s_job = -1;
    s_tab_rough = -1.0f;
  }
  for (;;) {
    if (threadIdx.x == 0) {
      long long tile = (long long)atomicAdd(counter, 1ULL);
      s_tile = tile;
      if (tile < total_tiles) {
        int k = find_range(begins, njobs, tile);
        if (k != s_job) {
          job = jobs[k];
          make_table(job.w, job.h, &tab);
          s_job = k;
        }
      }
    }
    __syncthreads();
    const long long tile = s_tile;
    if (tile >= total_tiles) break;
    const bool tabbed = tabulate && job.roughness != 0.0f;
    if (tabbed && job.roughness != s_tab_rough) {
      tabulate_hammersley(h_local, samples, job.roughness);
      __syncthreads();
      if (threadIdx.x == 0) s_tab_rough = job.roughness;
    }
    const long long local = tile - begins[s_job];
    const int x = (int)(local % job.tiles_x) * TX + (int)(threadIdx.x % TX);
    const int y = (int)(local / job.tiles_x) * TY + (int)(threadIdx.x / TX);
    if (x < job.ow && y < job.oh)
      job.out[(long long)y * job.pitch + x] =
          prefilter_texel(job.chain, tab, job.w, job.h, x, y, job.ow, job.oh, job.roughness,
                          samples, generator, tabbed ? h_local : nullptr);
    __syncthreads();  // before thread 0 rewrites the shared job for the next tile
  }
}

__global__ void __launch_bounds__(32 * kIrrWarps) batch_irradiance_partial_kernel(
    const IrrJob* __restrict__ jobs, const long long* __restrict__ begins, int njobs,
    float4* __restrict__ partial) {
  __shared__ ChainTable tab;
  __shared__ IrrJob job;
  __shared__ int s_job;
  __shared__ float cos_t[kThetaSamples], sin_t[kThetaSamples];
  __shared__ float band_smem[kBands][3];
  extern __shared__ float phi_table[];  // 2 * (max phi) floats
  if (threadIdx.x == 0) {
    int k = find_range(begins, njobs, blockIdx.x);
    s_job = k;
    job = jobs[k];
    make_table(job.w, job.h, &tab);
  }
  __syncthreads();
  float* cos_p = phi_table;
  float* sin_p = phi_table + job.phi;
  irradiance_tables(cos_t, sin_t, cos_p, sin_p, job.phi);
  __syncthreads();
  const long long local = (long long)blockIdx.x - begins[s_job];
  const long long texel = local / job.gb;
  const int gb = (int)(local % job.gb);
  const int count = kBands / job.gb;
  Float3 s = irradiance_block_bands(job.chain, tab, job.w, (int)(texel % job.ow),
                                    (int)(texel / job.ow), job.ow, job.oh, gb * count, count,
                                    job.phi, cos_t, sin_t, cos_p, sin_p, band_smem);
  if (threadIdx.x == 0)
    partial[job.partial_offset + texel * job.gb + gb] = make_float4(s.x, s.y, s.z, 0.0f);
}

__global__ void __launch_bounds__(256) batch_irradiance_finish_kernel(
    const IrrJob* __restrict__ jobs, const long long* __restrict__ texel_begins, int njobs,
    long long total_texels, const float4* __restrict__ partial) {
  long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= total_texels) return;
  const int k = find_range(texel_begins, njobs, g);
  const IrrJob& j = jobs[k];
  const long long texel = g - texel_begins[k];
  Float3 s = combine_partials(partial + j.partial_offset + texel * j.gb, j.gb);
  j.out[(texel / j.ow) * j.pitch + (texel % j.ow)] = irradiance_finish(s.x, s.y, s.z, j.phi);
}

// ---- tile shapes the tuner can pick -----------------------------------------
struct TileShape {
  int tx, ty;
};
constexpr TileShape kTileShapes[] = {{16, 8}, {32, 4}, {8, 8}, {16, 16}};
constexpr int kNumTileShapes = 4;
constexpr int kIrrTargets[] = {152 * 4, 152 * 8, 152 * 16};
constexpr int kNumIrrTargets = 3;

typedef void (*PfKernel)(const PfJob*, const long long*, int, long long, int, int, int,
                         unsigned long long*);

PfKernel pf_kernel_for(int s) {
  switch (s) {
    case 0: return batch_prefilter_kernel<16, 8>;
    case 1: return batch_prefilter_kernel<32, 4>;
    case 2: return batch_prefilter_kernel<8, 8>;
    default: return batch_prefilter_kernel<16, 16>;
  }
}

struct Choice {
  int shape = 0;
  int irr_target = 152 * 8;
};

std::mutex g_tune_mutex;
std::map<std::string, Choice>* g_tune_cache = nullptr;
bool g_tune_file_loaded = false;

void load_tune_file_locked() {
  if (g_tune_file_loaded) return;
  g_tune_file_loaded = true;
  const char* path = getenv("ALTHEA_IBL_TUNE_CACHE");
  if (!path) return;
  FILE* f = fopen(path, "r");
  if (!f) return;
  char key[4096];
  int tx, ty, irr;
  // Lines naming a tile shape or irradiance target this library does not have
  // (an edited or stale file) are skipped.
  while (fscanf(f, "%4095s %d %d %d", key, &tx, &ty, &irr) == 4) {
    bool known_irr = false;
    for (int t = 0; t < kNumIrrTargets; ++t) known_irr = known_irr || kIrrTargets[t] == irr;
    for (int s = 0; s < kNumTileShapes && known_irr; ++s)
      if (kTileShapes[s].tx == tx && kTileShapes[s].ty == ty) (*g_tune_cache)[key] = {s, irr};
  }
  fclose(f);
}

void append_tune_file_locked(const std::string& key, const Choice& c) {
  const char* path = getenv("ALTHEA_IBL_TUNE_CACHE");
  if (!path) return;
  FILE* f = fopen(path, "a");
  if (!f) return;
  fprintf(f, "%s %d %d %d\n", key.c_str(), kTileShapes[c.shape].tx, kTileShapes[c.shape].ty,
          c.irr_target);
  fclose(f);
}

}  // namespace
}  // namespace ibl

using namespace ibl;

struct althea_ibl_batch {
  int device = 0;
  int n = 0;
  althea_ibl_batch_params params{};
  // chain jobs, one group per level index
  std::vector<int> blit_level_jobs;    // jobs per level index
  std::vector<int> blit_level_blocks;  // blocks per level index
  BlitJob* d_blit = nullptr;           // all levels back to back
  long long* d_blit_begins = nullptr;
  // prefilter queue
  PfJob* d_pf = nullptr;
  long long* d_pf_begins = nullptr;
  int pf_jobs = 0;
  long long pf_tiles[kNumTileShapes] = {};
  std::vector<PfJob> h_pf;            // host copy (tiles_x depends on the shape)
  std::vector<std::vector<long long>> pf_begins;  // per shape
  unsigned long long* d_counter = nullptr;
  // irradiance
  IrrJob* d_irr = nullptr;
  long long* d_irr_begins = nullptr;
  long long* d_irr_texel_begins = nullptr;
  int irr_jobs = 0;
  long long irr_blocks = 0, irr_texels = 0;
  float4* d_partial = nullptr;
  size_t partial_bytes = 0;
  int max_phi = 0;
  std::vector<IrrJob> h_irr;
  // choice
  Choice choice;
  int tuned = 0;
  int persistent_blocks = 0;
  size_t pf_smem = 0;
  // graph
  cudaGraphExec_t exec = nullptr;
  cudaStream_t exec_stream = nullptr;
  int graph_kernels = -1;  // kernel nodes of the captured bake (-1: not captured)
  // precision path (ALTHEA_IBL_BATCH_PRECISION), after the shared chain
  // pass: the split passes of every probe, ONE persistent tcgen05
  // contraction over the work items of every probe and every probe's finish,
  // with the CUDA-core outputs on a side stream (joined back before the run
  // ends); a handful of launches in all.  Each probe has its own workspace:
  // all of their contractions are in flight at once.
  bool precision = false;
  cudaStream_t side = nullptr;
  cudaEvent_t fork_ev = nullptr, join_ev = nullptr;
  int out_format = ALTHEA_IBL_FORMAT_RGBA32F;
  std::vector<void*> tc_ws;   // one per probe
  ibl::TcBatch* tcb = nullptr;
};

namespace {

void free_batch(althea_ibl_batch* b) {
  if (!b) return;
  if (b->exec) cudaGraphExecDestroy(b->exec);
  cudaFree(b->d_blit);
  cudaFree(b->d_blit_begins);
  cudaFree(b->d_pf);
  cudaFree(b->d_pf_begins);
  cudaFree(b->d_counter);
  cudaFree(b->d_irr);
  cudaFree(b->d_irr_begins);
  cudaFree(b->d_irr_texel_begins);
  cudaFree(b->d_partial);
  tc_batch_destroy(b->tcb);
  for (void* p : b->tc_ws) cudaFree(p);
  if (b->side) cudaStreamDestroy(b->side);
  if (b->join_ev) cudaEventDestroy(b->join_ev);
  if (b->fork_ev) cudaEventDestroy(b->fork_ev);
  delete b;
}

// Uploads the irradiance job table for a split target (partial offsets move).
int build_irradiance(althea_ibl_batch* b, const althea_ibl_probe* probes, int target) {
  b->h_irr.clear();
  std::vector<long long> begins, tbegins;
  long long blocks = 0, texels = 0, poff = 0;
  long long total_texels = 0;
  for (int i = 0; i < b->n; ++i)
    if (probes[i].irradiance_dev)
      total_texels += (long long)probes[i].irradiance_width * probes[i].irradiance_height;
  for (int i = 0; i < b->n; ++i) {
    const althea_ibl_probe& p = probes[i];
    if (!p.irradiance_dev) continue;
    // The split is sized for the whole batch: each texel gets enough blocks
    // that the batch as a whole fills `target` blocks.
    IrrPlan pl = irr_plan(p.env_width, p.env_height,
                          p.irradiance_width, p.irradiance_height,
                          (int)std::max<long long>(
                              1, (long long)target * p.irradiance_width * p.irradiance_height /
                                     std::max<long long>(total_texels, 1)));
    IrrJob j;
    j.chain = reinterpret_cast<const float4*>(p.chain_dev);
    j.out = reinterpret_cast<float4*>(p.irradiance_dev);
    j.pitch = (long long)(p.irradiance_pitch_bytes / sizeof(float4));
    j.w = p.env_width;
    j.h = p.env_height;
    j.ow = p.irradiance_width;
    j.oh = p.irradiance_height;
    j.gb = pl.gb;
    j.phi = pl.phi;
    j.partial_offset = poff;
    begins.push_back(blocks);
    tbegins.push_back(texels);
    blocks += pl.texels * pl.gb;
    texels += pl.texels;
    poff += pl.texels * pl.gb;
    b->max_phi = std::max(b->max_phi, pl.phi);
    b->h_irr.push_back(j);
  }
  b->irr_jobs = (int)b->h_irr.size();
  b->irr_blocks = blocks;
  b->irr_texels = texels;
  if (b->irr_jobs == 0) return ALTHEA_IBL_OK;
  if (blocks > 0x7fffffffLL)
    return set_error(ALTHEA_IBL_ERR_UNSUPPORTED, "batched irradiance grid too large");
  size_t need = (size_t)poff * sizeof(float4);
  if (need > b->partial_bytes) {
    cudaFree(b->d_partial);
    b->d_partial = nullptr;
    cudaError_t e = cudaMalloc(&b->d_partial, need);
    if (e != cudaSuccess) return cuda_status(e, "batch irradiance workspace");
    b->partial_bytes = need;
  }
  cudaError_t e = cudaSuccess;
  if (!b->d_irr) e = cudaMalloc(&b->d_irr, sizeof(IrrJob) * b->irr_jobs);
  if (e == cudaSuccess && !b->d_irr_begins)
    e = cudaMalloc(&b->d_irr_begins, sizeof(long long) * b->irr_jobs);
  if (e == cudaSuccess && !b->d_irr_texel_begins)
    e = cudaMalloc(&b->d_irr_texel_begins, sizeof(long long) * b->irr_jobs);
  if (e == cudaSuccess)
    e = cudaMemcpy(b->d_irr, b->h_irr.data(), sizeof(IrrJob) * b->irr_jobs,
                   cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = cudaMemcpy(b->d_irr_begins, begins.data(), sizeof(long long) * b->irr_jobs,
                   cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = cudaMemcpy(b->d_irr_texel_begins, tbegins.data(), sizeof(long long) * b->irr_jobs,
                   cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda_status(e, "batch irradiance tables");
  size_t smem = 2 * (size_t)b->max_phi * sizeof(float);
  if (smem > 48 * 1024) {
    e = cudaFuncSetAttribute(batch_irradiance_partial_kernel,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return cuda_status(e, "irradiance smem attribute");
  }
  return ALTHEA_IBL_OK;
}

// Uploads the prefilter queue for tile shape s.
int select_shape(althea_ibl_batch* b, int s) {
  const int tx = kTileShapes[s].tx, ty = kTileShapes[s].ty;
  std::vector<PfJob> jobs = b->h_pf;
  std::vector<long long>& begins = b->pf_begins[s];
  for (auto& j : jobs) j.tiles_x = (j.ow + tx - 1) / tx;
  cudaError_t e = cudaMemcpy(b->d_pf, jobs.data(), sizeof(PfJob) * jobs.size(),
                             cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = cudaMemcpy(b->d_pf_begins, begins.data(), sizeof(long long) * begins.size(),
                   cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda_status(e, "batch prefilter tables");
  PfKernel k = pf_kernel_for(s);
  if (b->pf_smem > 48 * 1024) {
    e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)b->pf_smem);
    if (e != cudaSuccess) return cuda_status(e, "prefilter smem attribute");
  }
  int per_sm = 0, sms = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, tx * ty, b->pf_smem);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, b->device);
  if (e != cudaSuccess) return cuda_status(e, "prefilter occupancy");
  if (per_sm < 1) per_sm = 1;
  long long want = (long long)per_sm * sms;
  b->persistent_blocks = (int)std::min<long long>(want, std::max<long long>(b->pf_tiles[s], 1));
  b->choice.shape = s;
  return ALTHEA_IBL_OK;
}

int launch_chains(althea_ibl_batch* b, cudaStream_t st) {
  size_t job_off = 0;
  for (size_t l = 0; l < b->blit_level_jobs.size(); ++l) {
    int nj = b->blit_level_jobs[l], nb = b->blit_level_blocks[l];
    if (nj > 0 && nb > 0)
      batch_blit_kernel<<<nb, 256, 0, st>>>(b->d_blit + job_off, b->d_blit_begins + job_off, nj);
    job_off += nj;
  }
  return cuda_status(cudaGetLastError(), "batch chain launch");
}

int launch_prefilter_queue(althea_ibl_batch* b, cudaStream_t st) {
  const int s = b->choice.shape;
  if (b->pf_jobs == 0 || b->pf_tiles[s] == 0) return ALTHEA_IBL_OK;
  cudaError_t e = cudaMemsetAsync(b->d_counter, 0, sizeof(unsigned long long), st);
  if (e != cudaSuccess) return cuda_status(e, "queue reset");
  int tabulate = b->params.generator == ALTHEA_IBL_GEN_HAMMERSLEY &&
                 b->params.samples <= kMaxTabulatedSamples;
  pf_kernel_for(s)<<<b->persistent_blocks, kTileShapes[s].tx * kTileShapes[s].ty, b->pf_smem,
                     st>>>(b->d_pf, b->d_pf_begins, b->pf_jobs, b->pf_tiles[s],
                           b->params.samples, b->params.generator, tabulate, b->d_counter);
  return cuda_status(cudaGetLastError(), "batch prefilter launch");
}

int launch_irradiance_batch(althea_ibl_batch* b, cudaStream_t st) {
  if (b->irr_jobs == 0) return ALTHEA_IBL_OK;
  size_t smem = 2 * (size_t)b->max_phi * sizeof(float);
  batch_irradiance_partial_kernel<<<(unsigned)b->irr_blocks, 32 * kIrrWarps, smem, st>>>(
      b->d_irr, b->d_irr_begins, b->irr_jobs, b->d_partial);
  batch_irradiance_finish_kernel<<<(unsigned)((b->irr_texels + 255) / 256), 256, 0, st>>>(
      b->d_irr, b->d_irr_texel_begins, b->irr_jobs, b->irr_texels, b->d_partial);
  return cuda_status(cudaGetLastError(), "batch irradiance launch");
}

int launch_tc(althea_ibl_batch* b, cudaStream_t st) {
  return tc_batch_run(b->tcb, st, b->side, b->fork_ev, b->join_ev);
}

int launch_all(althea_ibl_batch* b, cudaStream_t st) {
  int r = launch_chains(b, st);
  if (b->precision) {
    if (!r) r = launch_tc(b, st);
  } else {
    if (!r) r = launch_prefilter_queue(b, st);
    if (!r) r = launch_irradiance_batch(b, st);
  }
  if (!r && b->params.lut_dev && b->params.lut_size > 0)
    r = launch_brdf_lut(b->params.lut_dev, b->params.lut_size, b->params.lut_pitch_bytes,
                        b->params.lut_samples, b->params.lut_orientation, st);
  return r;
}

std::string shape_key(const althea_ibl_probe* probes, int n, const althea_ibl_batch_params* p) {
  std::vector<std::string> parts;
  for (int i = 0; i < n; ++i) {
    std::ostringstream o;
    o << probes[i].env_width << 'x' << probes[i].env_height << ':'
      << probes[i].irradiance_width << 'x' << probes[i].irradiance_height << ':'
      << probes[i].mip_count;
    for (int m = 0; m < probes[i].mip_count; ++m)
      o << ',' << probes[i].mip_width[m] << 'x' << probes[i].mip_height[m];
    parts.push_back(o.str());
  }
  std::sort(parts.begin(), parts.end());
  std::map<std::string, int> counts;
  for (auto& s : parts) counts[s]++;
  std::ostringstream k;
  k << "n" << p->samples << "g" << p->generator;
  for (auto& kv : counts) k << '|' << kv.second << '*' << kv.first;
  return k.str();
}

float time_ms(cudaEvent_t a, cudaEvent_t b) {
  float ms = 0.0f;
  cudaEventElapsedTime(&ms, a, b);
  return ms;
}

int autotune(althea_ibl_batch* b, const althea_ibl_probe* probes, cudaStream_t st) {
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  int r = launch_chains(b, st);
  float best = 1e30f;
  int best_s = 0;
  for (int s = 0; s < kNumTileShapes && !r; ++s) {
    r = select_shape(b, s);
    if (r) break;
    r = launch_prefilter_queue(b, st);  // warm
    cudaEventRecord(e0, st);
    if (!r) r = launch_prefilter_queue(b, st);
    cudaEventRecord(e1, st);
    cudaEventSynchronize(e1);
    float ms = time_ms(e0, e1);
    if (ms < best) {
      best = ms;
      best_s = s;
    }
  }
  float best_i = 1e30f;
  int best_t = kIrrTargets[1];
  for (int t = 0; t < kNumIrrTargets && !r && b->irr_jobs > 0; ++t) {
    r = build_irradiance(b, probes, kIrrTargets[t]);
    if (r) break;
    r = launch_irradiance_batch(b, st);
    cudaEventRecord(e0, st);
    if (!r) r = launch_irradiance_batch(b, st);
    cudaEventRecord(e1, st);
    cudaEventSynchronize(e1);
    float ms = time_ms(e0, e1);
    if (ms < best_i) {
      best_i = ms;
      best_t = kIrrTargets[t];
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (r) return r;
  r = select_shape(b, best_s);
  if (!r) r = build_irradiance(b, probes, best_t);
  b->choice.irr_target = best_t;
  return r;
}

int check_probe(const althea_ibl_probe& p, int i, size_t texel) {
  int r = check_env(p.env_width, p.env_height);
  if (r) return r;
  if (!p.chain_dev || ((uintptr_t)p.chain_dev) % 16 ||
      (p.level0_dev && ((uintptr_t)p.level0_dev) % 16))
    return set_error(ALTHEA_IBL_ERR_INVALID_ARGUMENT, "probe %d: chain/level0 pointer", i);
  if (p.mip_count < 0 || p.mip_count > ALTHEA_IBL_MAX_MIPS)
    return set_error(ALTHEA_IBL_ERR_INVALID_ARGUMENT, "probe %d: mip_count %d", i, p.mip_count);
  for (int m = 0; m < p.mip_count; ++m) {
    r = check_image(p.mip_dev[m], p.mip_width[m], p.mip_height[m], p.mip_pitch_bytes[m], texel,
                    "batch mip");
    if (r) return r;
    if (!(p.mip_roughness[m] >= 0.0f && p.mip_roughness[m] <= 1.0f))
      return set_error(ALTHEA_IBL_ERR_INVALID_ARGUMENT, "probe %d mip %d roughness", i, m);
  }
  if (p.irradiance_dev) {
    r = check_irradiance_args(p.env_width, p.env_height, p.irradiance_width,
                              p.irradiance_height);
    if (!r)
      r = check_image(p.irradiance_dev, p.irradiance_width, p.irradiance_height,
                      p.irradiance_pitch_bytes, texel, "batch irradiance");
    if (r) return r;
  }
  return ALTHEA_IBL_OK;
}

}  // namespace

extern "C" int althea_ibl_batch_create(const althea_ibl_probe* probes, int n,
                                       const althea_ibl_batch_params* params, void* stream,
                                       althea_ibl_batch** out) {
  if (!out || !params || (n > 0 && !probes) || n < 0)
    return set_error(ALTHEA_IBL_ERR_INVALID_ARGUMENT, "null argument");
  *out = nullptr;
  if (params->samples < 1 || params->samples > (1 << 24) ||
      (params->generator != ALTHEA_IBL_GEN_REF_HASH &&
       params->generator != ALTHEA_IBL_GEN_HAMMERSLEY))
    return set_error(ALTHEA_IBL_ERR_INVALID_ARGUMENT, "samples/generator");
  if (params->lut_dev) {
    int r = check_image(params->lut_dev, params->lut_size, params->lut_size,
                        params->lut_pitch_bytes, 8, "batch lut");
    if (r) return r;
    if (params->lut_samples < 1 || params->lut_samples > (1 << 24) ||
        (params->lut_orientation != ALTHEA_IBL_LUT_ASSET &&
         params->lut_orientation != ALTHEA_IBL_LUT_CORRECTED))
      return set_error(ALTHEA_IBL_ERR_INVALID_ARGUMENT, "lut samples/orientation");
  }
  const bool precision = (params->flags & ALTHEA_IBL_BATCH_PRECISION) != 0;
  const bool half = (params->flags & ALTHEA_IBL_BATCH_HALF) != 0;
  if (half && !precision)
    return set_error(ALTHEA_IBL_ERR_UNSUPPORTED,
                     "RGBA16F batch outputs are produced by the precision path only");
  for (int i = 0; i < n; ++i) {
    int r = check_probe(probes[i], i, half ? 8 : 16);
    if (r) return r;
  }
  althea_ibl_batch* b = new (std::nothrow) althea_ibl_batch();
  if (!b) return set_error(ALTHEA_IBL_ERR_OUT_OF_MEMORY, "host allocation");
  b->n = n;
  b->params = *params;
  b->precision = precision;
  b->out_format = half ? ALTHEA_IBL_FORMAT_RGBA16F : ALTHEA_IBL_FORMAT_RGBA32F;
  cudaGetDevice(&b->device);
  cudaStream_t st = (cudaStream_t)stream;

  // ---- chain jobs, grouped by level index ---------------------------------
  std::vector<std::vector<BlitJob>> per_level(ALTHEA_IBL_MAX_LEVELS);
  for (int i = 0; i < n; ++i) {
    const althea_ibl_probe& p = probes[i];
    ChainTable t;
    make_table(p.env_width, p.env_height, &t);
    float4* c = reinterpret_cast<float4*>(p.chain_dev);
    if (!p.level0_dev) continue;  // chain supplied by the caller
    for (int l = 0; l < t.levels; ++l) {
      BlitJob j;
      j.copy = l == 0;
      j.src = l == 0 ? reinterpret_cast<const float4*>(p.level0_dev) : c + t.off[l - 1];
      j.dst = c + t.off[l];
      j.sw = l == 0 ? t.lw[0] : t.lw[l - 1];
      j.sh = l == 0 ? t.lh[0] : t.lh[l - 1];
      j.dw = t.lw[l];
      j.dh = t.lh[l];
      j.blocks_x = (j.dw + 31) / 32;
      per_level[l].push_back(j);
    }
  }
  std::vector<BlitJob> all_blit;
  std::vector<long long> all_blit_begins;
  for (int l = 0; l < ALTHEA_IBL_MAX_LEVELS; ++l) {
    long long blocks = 0;
    for (auto& j : per_level[l]) {
      all_blit.push_back(j);
      all_blit_begins.push_back(blocks);
      blocks += (long long)j.blocks_x * ((j.dh + 7) / 8);
    }
    if (!per_level[l].empty()) {
      b->blit_level_jobs.push_back((int)per_level[l].size());
      b->blit_level_blocks.push_back((int)blocks);
    }
  }
  // ---- precision path: one planned tensor-core bake per probe --------------
  if (precision) {
    // Lanes: longest-processing-time assignment by level-0 area.
    {
      cudaError_t e = cudaStreamCreateWithFlags(&b->side, cudaStreamNonBlocking);
      if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->fork_ev, cudaEventDisableTiming);
      if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->join_ev, cudaEventDisableTiming);
      if (e != cudaSuccess) {
        free_batch(b);
        return cuda_status(e, "precision side stream");
      }
    }
    std::vector<TcBatchProbe> tp(n);
    for (int i = 0; i < n; ++i) {
      const althea_ibl_probe& p = probes[i];
      TcBatchProbe& t = tp[i];
      t.chain = p.chain_dev;
      t.w = p.env_width;
      t.h = p.env_height;
      for (int m = 0; m < p.mip_count; ++m) {
        althea_ibl_mip_target mt;
        mt.out_dev = p.mip_dev[m];
        mt.pitch_bytes = p.mip_pitch_bytes[m];
        mt.width = p.mip_width[m];
        mt.height = p.mip_height[m];
        mt.roughness = p.mip_roughness[m];
        t.mips.push_back(mt);
      }
      t.irr = p.irradiance_dev;
      t.irr_w = p.irradiance_dev ? p.irradiance_width : 0;
      t.irr_h = p.irradiance_dev ? p.irradiance_height : 0;
      t.irr_pitch = p.irradiance_pitch_bytes;
      t.ws_bytes = tc_workspace_bytes(t.w, t.h, t.mips.data(), (int)t.mips.size(), nullptr,
                                      t.irr_w, t.irr_h, -1);
      if (t.ws_bytes == 0) {
        free_batch(b);
        return set_error(ALTHEA_IBL_ERR_UNSUPPORTED, "probe %d: precision plan: %s", i,
                         last_error());
      }
      void* ws = nullptr;
      cudaError_t e = cudaMalloc(&ws, t.ws_bytes);
      if (e != cudaSuccess) {
        free_batch(b);
        return cuda_status(e, "precision workspace");
      }
      b->tc_ws.push_back(ws);
      t.ws = ws;
    }
    int r = tc_batch_create(tp.data(), n, b->out_format, st, &b->tcb);
    if (r) {
      free_batch(b);
      return r;
    }
  }
  // ---- prefilter queue: full-sample jobs first, roughness 0 last ----------
  for (int pass = 0; pass < 2 && !precision; ++pass)
    for (int i = 0; i < n; ++i)
      for (int m = 0; m < probes[i].mip_count; ++m) {
        bool degenerate = probes[i].mip_roughness[m] == 0.0f;
        if ((pass == 0) == degenerate) continue;
        PfJob j;
        j.chain = reinterpret_cast<const float4*>(probes[i].chain_dev);
        j.out = reinterpret_cast<float4*>(probes[i].mip_dev[m]);
        j.pitch = (long long)(probes[i].mip_pitch_bytes[m] / sizeof(float4));
        j.w = probes[i].env_width;
        j.h = probes[i].env_height;
        j.ow = probes[i].mip_width[m];
        j.oh = probes[i].mip_height[m];
        j.roughness = probes[i].mip_roughness[m];
        j.tiles_x = 0;
        b->h_pf.push_back(j);
      }
  b->pf_jobs = (int)b->h_pf.size();
  b->pf_begins.assign(kNumTileShapes, {});
  for (int s = 0; s < kNumTileShapes; ++s) {
    long long tiles = 0;
    for (auto& j : b->h_pf) {
      b->pf_begins[s].push_back(tiles);
      tiles += (long long)((j.ow + kTileShapes[s].tx - 1) / kTileShapes[s].tx) *
               ((j.oh + kTileShapes[s].ty - 1) / kTileShapes[s].ty);
    }
    b->pf_tiles[s] = tiles;
  }
  b->pf_smem = (params->generator == ALTHEA_IBL_GEN_HAMMERSLEY &&
                params->samples <= kMaxTabulatedSamples)
                   ? 3 * (size_t)params->samples * sizeof(float)
                   : 0;

  cudaError_t e = cudaSuccess;
  size_t nb = std::max<size_t>(all_blit.size(), 1), np = std::max<size_t>(b->h_pf.size(), 1);
  e = cudaMalloc(&b->d_blit, sizeof(BlitJob) * nb);
  if (e == cudaSuccess) e = cudaMalloc(&b->d_blit_begins, sizeof(long long) * nb);
  if (e == cudaSuccess) e = cudaMalloc(&b->d_pf, sizeof(PfJob) * np);
  if (e == cudaSuccess) e = cudaMalloc(&b->d_pf_begins, sizeof(long long) * np);
  if (e == cudaSuccess) e = cudaMalloc(&b->d_counter, sizeof(unsigned long long));
  if (e == cudaSuccess && !all_blit.empty())
    e = cudaMemcpy(b->d_blit, all_blit.data(), sizeof(BlitJob) * all_blit.size(),
                   cudaMemcpyHostToDevice);
  if (e == cudaSuccess && !all_blit.empty())
    e = cudaMemcpy(b->d_blit_begins, all_blit_begins.data(),
                   sizeof(long long) * all_blit_begins.size(), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    free_batch(b);
    return cuda_status(e, "batch tables");
  }

  // ---- tile shape and split: cached choice, tuning, or the default -------
  std::string key = shape_key(probes, n, params);
  Choice cached;
  bool have = false;
  {
    std::lock_guard<std::mutex> lock(g_tune_mutex);
    if (!g_tune_cache) g_tune_cache = new std::map<std::string, Choice>();
    load_tune_file_locked();
    auto it = g_tune_cache->find(key);
    if (it != g_tune_cache->end()) {
      cached = it->second;
      have = true;
    }
  }
  int r = ALTHEA_IBL_OK;
  if (precision) {
    r = select_shape(b, 0);  // fixed tensor-core tiles: nothing to tune
  } else if (have) {
    r = select_shape(b, cached.shape);
    if (!r) r = build_irradiance(b, probes, cached.irr_target);
    b->choice.irr_target = cached.irr_target;
    b->tuned = 1;
  } else if (params->flags & ALTHEA_IBL_BATCH_AUTOTUNE) {
    r = autotune(b, probes, st);
    if (!r) {
      b->tuned = 1;
      std::lock_guard<std::mutex> lock(g_tune_mutex);
      (*g_tune_cache)[key] = b->choice;
      append_tune_file_locked(key, b->choice);
    }
  } else {
    r = select_shape(b, 0);
    if (!r) r = build_irradiance(b, probes, kIrrTargets[1]);
    b->choice.irr_target = kIrrTargets[1];
  }
  if (r) {
    free_batch(b);
    return r;
  }
  *out = b;
  return ALTHEA_IBL_OK;
}

extern "C" int althea_ibl_batch_run(althea_ibl_batch* b, void* stream) {
  ibl::NvtxRange nvtx_range("althea_ibl_batch_run");
  if (!b) return set_error(ALTHEA_IBL_ERR_INVALID_ARGUMENT, "null batch");
  cudaStream_t st = (cudaStream_t)stream;
  const bool want_graph = (b->params.flags & ALTHEA_IBL_BATCH_GRAPH) && st != nullptr;
  if (!want_graph) return launch_all(b, st);
  if (b->exec && b->exec_stream == st) {
    cudaError_t e = cudaGraphLaunch(b->exec, st);
    return cuda_status(e, "batch graph launch");
  }
  if (b->exec) {
    cudaGraphExecDestroy(b->exec);
    b->exec = nullptr;
  }
  cudaError_t e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return cuda_status(e, "batch graph capture");
  int r = launch_all(b, st);
  cudaGraph_t graph = nullptr;
  e = cudaStreamEndCapture(st, &graph);
  if (r) {
    if (graph) cudaGraphDestroy(graph);
    return r;
  }
  if (e != cudaSuccess) return cuda_status(e, "batch graph capture end");
  size_t nodes = 0;
  if (cudaGraphGetNodes(graph, nullptr, &nodes) == cudaSuccess && nodes > 0) {
    std::vector<cudaGraphNode_t> list(nodes);
    int kernels = 0;
    if (cudaGraphGetNodes(graph, list.data(), &nodes) == cudaSuccess) {
      for (size_t i = 0; i < nodes; ++i) {
        cudaGraphNodeType t;
        if (cudaGraphNodeGetType(list[i], &t) == cudaSuccess && t == cudaGraphNodeTypeKernel)
          ++kernels;
      }
      b->graph_kernels = kernels;
    }
  }
  e = cudaGraphInstantiate(&b->exec, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) {
    b->exec = nullptr;
    return cuda_status(e, "batch graph instantiate");
  }
  b->exec_stream = st;
  return cuda_status(cudaGraphLaunch(b->exec, st), "batch graph launch");
}

extern "C" int althea_ibl_batch_describe(const althea_ibl_batch* b, althea_ibl_batch_info* info) {
  if (!b || !info) return set_error(ALTHEA_IBL_ERR_INVALID_ARGUMENT, "null argument");
  info->probes = b->n;
  info->prefilter_jobs = b->pf_jobs;
  info->prefilter_tiles = (int)b->pf_tiles[b->choice.shape];
  info->irradiance_blocks = (int)b->irr_blocks;
  info->tile_x = kTileShapes[b->choice.shape].tx;
  info->tile_y = kTileShapes[b->choice.shape].ty;
  info->persistent_blocks = b->persistent_blocks;
  info->irradiance_target_blocks = b->choice.irr_target;
  info->tuned = b->tuned;
  info->graph = b->exec != nullptr;
  info->graph_kernels = b->exec ? b->graph_kernels : -1;
  info->contraction_items = b->tcb ? tc_batch_items(b->tcb) : 0;
  return ALTHEA_IBL_OK;
}

extern "C" int althea_ibl_batch_status(const althea_ibl_batch* b, void* stream) {
  if (!b) return set_error(ALTHEA_IBL_ERR_INVALID_ARGUMENT, "null batch");
  cudaStream_t st = (cudaStream_t)stream;
  if (b->tcb) return tc_batch_error(b->tcb, st);
  return cuda_status(cudaStreamSynchronize(st), "batch status");
}

extern "C" int althea_ibl_batch_destroy(althea_ibl_batch* b) {
  free_batch(b);
  return ALTHEA_IBL_OK;
}
