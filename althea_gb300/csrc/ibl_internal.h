// ibl_internal.h -- declarations shared between the translation units of
// libalthea_ibl.so (not part of the public C ABI).
#pragma once

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <cstddef>
#include <vector>

#include "althea_ibl.h"

namespace ibl {

// An NVTX range around a public call (header-only NVTX3: without a profiler
// attached the push and pop return at once).  Profilers show the library's
// stages on the host timeline under these names.
struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange&) = delete;
  NvtxRange& operator=(const NvtxRange&) = delete;
};

struct IrrPlan {
  int phi;             // int(300 * H / W)
  long long texels;    // output texels
  int gb;              // 256-thread blocks per output texel
  size_t workspace;    // texels * gb partial sums (float4)
};

int set_error(int status, const char* fmt, ...);
int cuda_status(cudaError_t e, const char* what);
const char* last_error();

int check_env(int w, int h);
int check_image(const void* p, int w, int h, size_t pitch, size_t texel_bytes, const char* what);
int check_irradiance_args(int w, int h, int ow, int oh);
// target_blocks: how many 256-thread blocks the split should aim for
// (<= 0: 8 per SM of a 152-SM GB300).
IrrPlan irr_plan(int w, int h, int ow, int oh, int target_blocks = 0);

int launch_build_chain(const float* level0, int w, int h, float* chain, cudaStream_t st);
int launch_prefilter(const float* chain, int w, int h, const althea_ibl_mip_target* mips,
                     int mip_count, int samples, int generator, cudaStream_t st);
int launch_irradiance(const float* chain, int w, int h, float* out, int ow, int oh,
                      size_t pitch_bytes, void* ws, cudaStream_t st);
// Roughness-0 mip as the single reflected sample (no Monte Carlo accumulation);
// out_half: RGBA16F output (8-byte texels) instead of RGBA32F.
int launch_delta_mip(const float* chain, int w, int h, const althea_ibl_mip_target* mip,
                     int out_half, cudaStream_t st);
// Delta mips of many probes in one launch (ibl_plain.cu): job k covers
// blocks [begins[k], begins[k + 1]) of 32 x 8 texels, blocks_x per row.
struct DeltaJob {
  const float* chain;
  int w, h;
  void* out;
  long long pitch;  // texels
  int ow, oh, out_half, blocks_x;
};
int launch_delta_batch(const DeltaJob* d_jobs, const long long* d_begins, int njobs,
                       long long blocks, cudaStream_t st);

// A second stream for work that does not feed the tensor-core contractions
// (the outputs summed on the CUDA cores): forked from the bake's stream after
// the direction tables with `fork`, joined back with `join` before the bake
// returns, so the CUDA-core kernels can share SMs with the tensor-bound ones.
struct SideStream {
  cudaStream_t stream;
  cudaEvent_t fork, join;
};

// Precision path (ibl_tc.cu): the bake behind althea_ibl_bake_tc_ex, and its
// workspace size (0 when the plan is unsupported).  side may be null (one
// stream).  tables = false: the workspace already holds this plan's direction
// tables and windows (they depend on the sizes only), from an earlier bake
// ordered before this one.  timing, when not null, is a pair of timing events
// recorded on `stream` just before and just after the contraction launch.
int tc_bake(const float* chain, int w, int h, const althea_ibl_mip_target* mips, int n,
            const int* levels, float* irr_out, int irr_w, int irr_h, size_t irr_pitch,
            int irr_level, void* ws, size_t ws_bytes, int out_format, cudaStream_t stream,
            const SideStream* side = nullptr, bool tables = true,
            const cudaEvent_t* timing = nullptr);
size_t tc_workspace_bytes(int w, int h, const althea_ibl_mip_target* mips, int n,
                          const int* levels, int irr_w, int irr_h, int irr_level);

// Precision batches (ibl_tc.cu): every probe planned with the planner's
// levels into its own workspace, its tables computed once at creation.  A
// run launches the split passes of every probe (one launch), ONE persistent
// contraction kernel over a queue of (job, row tile, column block, split)
// work items of every probe, then every probe's finish (one launch); the
// narrow outputs and roughness-0 mips go to `side` beside them (one launch
// each).  The results equal the probes' single bakes.
struct TcBatchProbe {
  const float* chain;
  int w, h;
  std::vector<althea_ibl_mip_target> mips;
  float* irr;  // may be null
  int irr_w, irr_h;
  size_t irr_pitch;
  void* ws;    // tc_workspace_bytes of this probe, 256-byte aligned
  size_t ws_bytes;
};
struct TcBatch;
// Builds the plan and the device job tables, and computes every probe's
// tables on `st` (synchronised before it returns).
int tc_batch_create(const TcBatchProbe* probes, int n, int out_format, cudaStream_t st,
                    TcBatch** out);
int tc_batch_run(TcBatch* b, cudaStream_t st, cudaStream_t side, cudaEvent_t fork_ev,
                 cudaEvent_t join_ev);
int tc_batch_items(const TcBatch* b);
// Synchronises `st` and reports a work item whose bounded wait gave up.
int tc_batch_error(const TcBatch* b, cudaStream_t st);
void tc_batch_destroy(TcBatch* b);
int launch_brdf_lut(float* out, int n, size_t pitch_bytes, int samples, int orientation,
                    cudaStream_t st);
// Sun lobes added to an env level 0 (ibl_suns.cu); out may equal base.
int launch_apply_suns(const float* base, float* out, int w, int h, const althea_ibl_sun* suns,
                      int n, cudaStream_t st);
// Reflection-buffer convolution (ibl_ssr.cu): levels 1..mips-1 from level 0.
int ssr_convolve(void* const* levels, const size_t* pitch_bytes, int w, int h, int mips,
                 cudaStream_t st);

}  // namespace ibl
