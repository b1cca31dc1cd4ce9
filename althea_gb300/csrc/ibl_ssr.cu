// ibl_ssr.cu -- glossy convolution of the reflection buffer's mip chain.
//
// Restates Shaders/SSRGlossyConvolve.comp:25-53 as dispatched by
// ReflectionBuffer::convolveReflectionBuffer (Src/ReflectionBuffer.cpp:163-275):
// the RGBA16F reflection buffer (Src/ReflectionBuffer.cpp:28-36, 5 mips at the
// swapchain extent) keeps the screen-space reflections in level 0, and every
// level l >= 1 is a 7-tap Gaussian of level l-1 along (0,1) for odd l and
// (1,0) for even l.  The taps read level l-1 through a one-level view with the
// default sampler (LINEAR, CLAMP_TO_EDGE; Src/ReflectionBuffer.cpp:62-75) at
// uv = texelPos / (w_l, h_l), offsets divided by w_l in both directions.
//
// Arithmetic is the shader's, in FP32 without contraction (this unit is built
// with -fmad=false and uses the _rn intrinsics, which are never fused): the
// bilinear sample is ((w00 t00 + w10 t10) + w01 t01) + w11 t11 with the Vulkan
// weights, the taps are accumulated left to right from 0, and the store rounds
// to binary16 to nearest even -- so results are bit-identical to the CPU
// restatement of the shader.
//
// One kernel per level (levels depend on each other), launched with
// programmatic stream serialisation: a level's blocks are resident and have
// their coordinates ready when the level before it completes.  Each thread
// owns one output texel.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "althea_ibl.h"
#include "ibl_internal.h"

namespace {

// The Gaussian (SSRGlossyConvolve.comp:42-51): offsets in texels of level l
// and their weights, as FP32 literals like the shader's.
constexpr float kOff1 = 1.411764705882353f, kOff2 = 3.2941176470588234f,
                kOff3 = 5.176470588235294f;
constexpr float kW0 = 0.1964825501511404f, kW1 = 0.2969069646728344f,
                kW2 = 0.09447039785044732f, kW3 = 0.010381362401148057f;

constexpr int kBlockX = 32, kBlockY = 8;
constexpr int kMaxLevels = 16;

struct Level {
  const uint2* src;  // level l-1, one uint2 (4 halfs) per texel
  uint2* dst;        // level l
  long long src_pitch, dst_pitch;  // in texels
  int sw, sh, dw, dh;
  float q1, q2, q3;  // offsets / resolution: kOff_k / (float)dw (IEEE division, on the host)
};

__device__ __forceinline__ float2 halves(uint32_t v) {
  return __half22float2(*reinterpret_cast<const __half2*>(&v));
}

__device__ __forceinline__ float2 splat(float v) { return make_float2(v, v); }

// Channel pairs, each product and sum rounded on its own (__fmul_rn/__fadd_rn
// are never fused into a multiply-add).  Packed FP32x2 products feeding packed
// FP32x2 sums (written as mul/add.rn.f32x2, or as FFMA2 with a -0 addend /
// unit multiplier) gave results one unit in the last place away on rare
// texels -- a product and the sum after it evidently became one fused
// operation.  Packed products alone, or packed sums alone, were exact but no
// faster (the kernel is bound by loads and conversions), so the scalar forms
// stay.
__device__ __forceinline__ float2 mul2(float2 a, float2 b) {
  return make_float2(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y));
}
__device__ __forceinline__ float2 add2(float2 a, float2 b) {
  return make_float2(__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y));
}

// Bilinear footprint along one axis: x = p * size - 0.5, the two clamped
// indices and the fraction (Vulkan spec, LINEAR + CLAMP_TO_EDGE).
struct Axis {
  int i0, i1;
  float frac;
};

__device__ __forceinline__ Axis axis(float p, int size) {
  const float x = __fsub_rn(__fmul_rn(p, (float)size), 0.5f);
  const float fx = floorf(x);
  Axis r;
  r.frac = __fsub_rn(x, fx);
  const int i = (int)fx;
  r.i0 = min(max(i, 0), size - 1);
  r.i1 = min(max(i + 1, 0), size - 1);
  return r;
}

// acc += textureLod(src, (u, v)) * kw for one tap whose footprint is (ax, ay).
__device__ __forceinline__ void tap(const Level& L, const Axis& ax, const Axis& ay, float kw,
                                    float2& acc_rg, float2& acc_ba) {
  const float a = ax.frac, b = ay.frac;
  const float oa = __fsub_rn(1.0f, a), ob = __fsub_rn(1.0f, b);
  const float2 w00 = splat(__fmul_rn(oa, ob)), w10 = splat(__fmul_rn(a, ob));
  const float2 w01 = splat(__fmul_rn(oa, b)), w11 = splat(__fmul_rn(a, b));
  const uint2* r0 = L.src + (long long)ay.i0 * L.src_pitch;
  const uint2* r1 = L.src + (long long)ay.i1 * L.src_pitch;
  const uint2 t00 = __ldg(r0 + ax.i0), t10 = __ldg(r0 + ax.i1);
  const uint2 t01 = __ldg(r1 + ax.i0), t11 = __ldg(r1 + ax.i1);
  float2 rg = mul2(w00, halves(t00.x));
  float2 ba = mul2(w00, halves(t00.y));
  rg = add2(rg, mul2(w10, halves(t10.x)));
  ba = add2(ba, mul2(w10, halves(t10.y)));
  rg = add2(rg, mul2(w01, halves(t01.x)));
  ba = add2(ba, mul2(w01, halves(t01.y)));
  rg = add2(rg, mul2(w11, halves(t11.x)));
  ba = add2(ba, mul2(w11, halves(t11.y)));
  const float2 k = splat(kw);
  acc_rg = add2(acc_rg, mul2(rg, k));
  acc_ba = add2(acc_ba, mul2(ba, k));
}

// VERT: direction (0, 1) (odd levels); else (1, 0).
template <bool VERT>
__global__ void __launch_bounds__(kBlockX* kBlockY) ssr_level_kernel(Level L) {
  // Let the next level's blocks be scheduled as this grid's retire; they wait
  // for this grid's completion before reading what it writes.
  asm volatile("griddepcontrol.launch_dependents;");
  const int x = blockIdx.x * kBlockX + threadIdx.x;
  const int y = blockIdx.y * kBlockY + threadIdx.y;
  const bool live = x < L.dw && y < L.dh;
  // texelUv; the offsets / resolution (resolution = the level's width) come in L
  const float u = __fdiv_rn((float)x, (float)L.dw);
  const float v = __fdiv_rn((float)y, (float)L.dh);
  const float q1 = L.q1, q2 = L.q2, q3 = L.q3;
  // The level before this one was written by the previous launch.
  asm volatile("griddepcontrol.wait;" ::: "memory");
  float2 rg = make_float2(0.0f, 0.0f), ba = make_float2(0.0f, 0.0f);
  if (VERT) {
    // A warp is one output row, so the seven row footprints are the same on
    // every lane: lanes 0-6 compute one tap each and the warp shares them.
    if (y >= L.dh) return;  // the whole warp
    const int lane = threadIdx.x, k = lane < 7 ? lane : 0;
    const float d = k == 0 ? 0.0f : (k <= 2 ? q1 : (k <= 4 ? q2 : q3));
    const float p = k == 0 ? v : ((k & 1) ? __fadd_rn(v, d) : __fsub_rn(v, d));
    const Axis mine = axis(p, L.sh);
    Axis m[7];
#pragma unroll
    for (int t = 0; t < 7; ++t) {
      m[t].i0 = __shfl_sync(0xffffffffu, mine.i0, t);
      m[t].i1 = __shfl_sync(0xffffffffu, mine.i1, t);
      m[t].frac = __shfl_sync(0xffffffffu, mine.frac, t);
    }
    if (x >= L.dw) return;
    const Axis ax = axis(u, L.sw);
    tap(L, ax, m[0], kW0, rg, ba);
    tap(L, ax, m[1], kW1, rg, ba);
    tap(L, ax, m[2], kW1, rg, ba);
    tap(L, ax, m[3], kW2, rg, ba);
    tap(L, ax, m[4], kW2, rg, ba);
    tap(L, ax, m[5], kW3, rg, ba);
    tap(L, ax, m[6], kW3, rg, ba);
  } else {
    if (!live) return;
    const Axis ay = axis(v, L.sh);
    tap(L, axis(u, L.sw), ay, kW0, rg, ba);
    tap(L, axis(__fadd_rn(u, q1), L.sw), ay, kW1, rg, ba);
    tap(L, axis(__fsub_rn(u, q1), L.sw), ay, kW1, rg, ba);
    tap(L, axis(__fadd_rn(u, q2), L.sw), ay, kW2, rg, ba);
    tap(L, axis(__fsub_rn(u, q2), L.sw), ay, kW2, rg, ba);
    tap(L, axis(__fadd_rn(u, q3), L.sw), ay, kW3, rg, ba);
    tap(L, axis(__fsub_rn(u, q3), L.sw), ay, kW3, rg, ba);
  }
  const __half2 o_rg = __floats2half2_rn(rg.x, rg.y), o_ba = __floats2half2_rn(ba.x, ba.y);
  uint2 o;
  o.x = *reinterpret_cast<const uint32_t*>(&o_rg);
  o.y = *reinterpret_cast<const uint32_t*>(&o_ba);
  L.dst[(long long)y * L.dst_pitch + x] = o;
}

int dim(int d, int l) {
  const int v = d >> l;
  return v < 1 ? 1 : v;
}

int launch_level(const Level& L, bool vert, cudaStream_t st) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)((L.dw + kBlockX - 1) / kBlockX),
                     (unsigned)((L.dh + kBlockY - 1) / kBlockY), 1);
  cfg.blockDim = dim3(kBlockX, kBlockY, 1);
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cudaError_t e = vert ? cudaLaunchKernelEx(&cfg, ssr_level_kernel<true>, L)
                       : cudaLaunchKernelEx(&cfg, ssr_level_kernel<false>, L);
  return ibl::cuda_status(e, "ssr convolution launch");
}

}  // namespace

namespace ibl {

int ssr_convolve(void* const* levels, const size_t* pitch_bytes, int w, int h, int mips,
                 cudaStream_t st) {
  if (w < 1 || h < 1 || w > 65536 || h > 65536)
    return set_error(ALTHEA_IBL_ERR_INVALID_ARGUMENT, "ssr: bad size %dx%d", w, h);
  if (mips < 1 || mips > kMaxLevels)
    return set_error(ALTHEA_IBL_ERR_INVALID_ARGUMENT, "ssr: mip_count %d not in 1..%d", mips,
                     kMaxLevels);
  for (int l = 0; l < mips; ++l) {
    const int st_ = check_image(levels[l], dim(w, l), dim(h, l), pitch_bytes[l], 8, "ssr level");
    if (st_ != ALTHEA_IBL_OK) return st_;
  }
  for (int l = 1; l < mips; ++l) {
    Level L;
    L.src = static_cast<const uint2*>(levels[l - 1]);
    L.dst = static_cast<uint2*>(levels[l]);
    L.src_pitch = (long long)(pitch_bytes[l - 1] / 8);
    L.dst_pitch = (long long)(pitch_bytes[l] / 8);
    L.sw = dim(w, l - 1);
    L.sh = dim(h, l - 1);
    L.dw = dim(w, l);
    L.dh = dim(h, l);
    const float res = (float)L.dw;  // resolution = the level's width
    L.q1 = kOff1 / res;
    L.q2 = kOff2 / res;
    L.q3 = kOff3 / res;
    const int s = launch_level(L, (l & 1) != 0, st);
    if (s != ALTHEA_IBL_OK) return s;
  }
  return ALTHEA_IBL_OK;
}

}  // namespace ibl

extern "C" {

size_t althea_ssr_level_offset(int width, int height, int level) {
  if (width < 1 || height < 1 || level < 0) return 0;
  size_t off = 0;
  for (int l = 0; l < level; ++l) off += (size_t)dim(width, l) * (size_t)dim(height, l);
  return off;
}

int althea_ssr_convolve_levels(void* const* levels_dev, const size_t* pitch_bytes, int width,
                               int height, int mip_count, void* stream) {
  if (!levels_dev || !pitch_bytes)
    return ibl::set_error(ALTHEA_IBL_ERR_INVALID_ARGUMENT, "ssr: null level arrays");
  return ibl::ssr_convolve(levels_dev, pitch_bytes, width, height, mip_count,
                           static_cast<cudaStream_t>(stream));
}

int althea_ssr_convolve(void* chain_dev, int width, int height, int mip_count, void* stream) {
  if (mip_count < 1 || mip_count > kMaxLevels)
    return ibl::set_error(ALTHEA_IBL_ERR_INVALID_ARGUMENT, "ssr: mip_count %d not in 1..%d",
                          mip_count, kMaxLevels);
  if (width < 1 || height < 1)
    return ibl::set_error(ALTHEA_IBL_ERR_INVALID_ARGUMENT, "ssr: bad size %dx%d", width, height);
  void* lv[kMaxLevels];
  size_t pitch[kMaxLevels];
  for (int l = 0; l < mip_count; ++l) {
    lv[l] = chain_dev ? static_cast<char*>(chain_dev) + 8 * althea_ssr_level_offset(width, height, l)
                      : nullptr;
    pitch[l] = (size_t)dim(width, l) * 8;
  }
  return ibl::ssr_convolve(lv, pitch, width, height, mip_count, static_cast<cudaStream_t>(stream));
}

}  // extern "C"
