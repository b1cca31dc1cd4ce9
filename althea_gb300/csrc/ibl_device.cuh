// ibl_device.cuh -- device-side building blocks of the plain IBL path:
// env-chain level table, the Vulkan trilinear REPEAT sampler, direction
// mapping, the reference's hash RNG and GGX sampling.
//
// This translation unit family is compiled with -fmad=false: every float
// expression below is evaluated as separate IEEE-754 single operations in the
// order written (which is the left-to-right order of the reference GLSL), and
// the transcendental built-ins come from glsl_builtins.h, so results match the
// CPU oracle bit for bit.
#pragma once

#include <cstdint>

#include "glsl_builtins.h"

namespace ibl {

constexpr float kPi = 3.14159265359f;  // PreFilterEnvMap.comp:4 (GLSL float literal)
constexpr int kMaxLevels = 16;

struct Float3 {
  float x, y, z;
};

__device__ __forceinline__ Float3 f3(float x, float y, float z) { return Float3{x, y, z}; }

// Level table of a packed RGBA32F chain.  Kept in shared memory by the
// kernels: lanes index it with divergent level numbers.
struct ChainTable {
  int levels;
  int lw[kMaxLevels];
  int lh[kMaxLevels];
  long long off[kMaxLevels];  // in texels
};

__host__ __device__ inline int level_dim(int d, int l) {
  int v = d >> l;
  return v < 1 ? 1 : v;
}

// Src/Utilities.cpp:97-100: 1 + floor(log2(max(w, h))), computed exactly on
// integers (floor(log2(n)) is the index of the top set bit).
__host__ __device__ inline int chain_levels(int w, int h) {
  unsigned m = (unsigned)(w > h ? w : h);
  int l = 0;
  while (m > 1u) {
    m >>= 1;
    ++l;
  }
  return 1 + l;
}

__host__ __device__ inline void make_table(int w, int h, ChainTable* t) {
  t->levels = chain_levels(w, h);
  long long off = 0;
  for (int l = 0; l < kMaxLevels; ++l) {
    int lw = level_dim(w, l), lh = level_dim(h, l);
    t->lw[l] = lw;
    t->lh[l] = lh;
    t->off[l] = off;
    if (l < t->levels) off += (long long)lw * lh;
  }
}

// Job tables of batched launches: the index of the last range whose begin
// <= key (begins ascending, begins[0] = 0), so block b of a launch belongs to
// job find_range(begins, n, b) as its block b - begins[job].
__device__ __forceinline__ int find_range(const long long* __restrict__ begins, int n,
                                          long long key) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (begins[mid] <= key)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

// Index wrap for REPEAT.  Texel coordinates normally lie in [-1, n]; the
// general branch keeps any input (even from NaN) in bounds.
__device__ __forceinline__ int wrap_repeat(int i, int n) {
  int r = i < 0 ? i + n : i;  // -1 -> n-1
  r = r >= n ? r - n : r;     // n -> 0
  if ((unsigned)r >= (unsigned)n) {
    r = i % n;
    r = r < 0 ? r + n : r;
  }
  return r;
}

__device__ __forceinline__ float4 ldg4(const float4* p) { return __ldg(p); }

// Bilinear combination ((w00*t00 + w10*t10) + w01*t01) + w11*t11 (the order
// used by the oracle), returned for rgb only.
__device__ __forceinline__ Float3 bilerp3(float4 t00, float4 t10, float4 t01, float4 t11, float a,
                                          float b) {
  float w00 = (1.0f - a) * (1.0f - b);
  float w10 = a * (1.0f - b);
  float w01 = (1.0f - a) * b;
  float w11 = a * b;
  return f3(((w00 * t00.x + w10 * t10.x) + w01 * t01.x) + w11 * t11.x,
            ((w00 * t00.y + w10 * t10.y) + w01 * t01.y) + w11 * t11.y,
            ((w00 * t00.z + w10 * t10.z) + w01 * t01.z) + w11 * t11.z);
}

__device__ __forceinline__ Float3 sample_level(const float4* __restrict__ chain,
                                               const ChainTable& t, int l, float u, float v) {
  int lw = t.lw[l], lh = t.lh[l];
  const float4* img = chain + t.off[l];
  float x = u * (float)lw - 0.5f;
  float y = v * (float)lh - 0.5f;
  float fx = floorf(x), fy = floorf(y);
  float a = x - fx, b = y - fy;
  int ix = (int)fx, iy = (int)fy;
  int i0 = wrap_repeat(ix, lw), i1 = wrap_repeat(ix + 1, lw);
  int j0 = wrap_repeat(iy, lh), j1 = wrap_repeat(iy + 1, lh);
  const float4* r0 = img + (long long)j0 * lw;
  const float4* r1 = img + (long long)j1 * lw;
  float4 t00 = ldg4(r0 + i0), t10 = ldg4(r0 + i1);
  float4 t01 = ldg4(r1 + i0), t11 = ldg4(r1 + i1);
  return bilerp3(t00, t10, t01, t11, a, b);
}

// textureLod with the precompute sampler (REPEAT/LINEAR/LINEAR, maxLod =
// levels-1; Src/ImageBasedLighting.cpp:168-174, Src/Sampler.cpp:90-113).
__device__ __forceinline__ Float3 texture_lod(const float4* __restrict__ chain,
                                              const ChainTable& t, float u, float v, float lod) {
  int q = t.levels - 1;
  float lam = lod;
  if (lam < 0.0f) lam = 0.0f;
  if (lam > (float)q) lam = (float)q;
  float fl = floorf(lam);
  int l0 = (int)fl;
  if (l0 < 0) l0 = 0;  // only reachable for NaN lod
  if (l0 > q) l0 = q;
  float d = lam - fl;
  Float3 lo = sample_level(chain, t, l0, u, v);
  if (d > 0.0f) {
    int l1 = l0 + 1 > q ? q : l0 + 1;
    Float3 hi = sample_level(chain, t, l1, u, v);
    lo = f3((1.0f - d) * lo.x + d * hi.x, (1.0f - d) * lo.y + d * hi.y,
            (1.0f - d) * lo.z + d * hi.z);
  }
  return lo;
}

// sampleEnvMap (PreFilterEnvMap.comp:98-122, GenIrradianceMap.comp:78-102).
__device__ __forceinline__ Float3 sample_env(const float4* __restrict__ chain,
                                             const ChainTable& t, Float3 dir, float mip) {
  float pitch = 0.0f, yaw = 0.0f;
  float len_xz = sqrtf(dir.x * dir.x + dir.z * dir.z);
  if (len_xz > 0.001f) {
    yaw = agb_atan2(dir.z, dir.x);
    pitch = agb_atan(dir.y / len_xz);
  } else if (dir.y > 0.0f) {
    pitch = 0.5f * kPi;
  } else {
    pitch = -0.5f * kPi;
  }
  // yaw / (2.0 * PI) + 0.5 and pitch / PI + 0.5, with the IEEE quotients
  // formed from the correctly rounded constant reciprocals.
  float u = agb_div_rcp(yaw, 2.0f * kPi, AGB_RCP_TWO_PI_F) + 0.5f;
  float v = agb_div_rcp(pitch, kPi, AGB_RCP_PI_F) + 0.5f;
  return texture_lod(chain, t, u, v, mip);
}

// Texel-corner direction (PreFilterEnvMap.comp:128-134).
__device__ __forceinline__ Float3 texel_dir(int x, int y, int ow, int oh) {
  float u = (float)x / (float)ow;
  float v = (float)y / (float)oh;
  float yaw = kPi * (2.0f * u - 1.0f);
  float pitch = kPi * (v - 0.5f);
  float sp, cp, sy, cy;
  agb_sincos(pitch, &sp, &cp);
  agb_sincos(yaw, &sy, &cy);
  return f3(cp * cy, sp, cp * sy);
}

// coordinateSystem / LocalToWorld (PreFilterEnvMap.comp:22-34).
__device__ __forceinline__ void local_frame(Float3 n, Float3& t, Float3& b) {
  if (agb_abs(n.x) > agb_abs(n.y)) {
    float s = sqrtf(n.x * n.x + n.z * n.z);
    t = f3(-n.z / s, 0.0f / s, n.x / s);
  } else {
    float s = sqrtf(n.y * n.y + n.z * n.z);
    t = f3(0.0f / s, n.z / s, -n.y / s);
  }
  b = f3(n.y * t.z - n.z * t.y, n.z * t.x - n.x * t.z, n.x * t.y - n.y * t.x);
}

__device__ __forceinline__ Float3 to_world(Float3 t, Float3 b, Float3 n, Float3 v) {
  return f3((t.x * v.x + b.x * v.y) + n.x * v.z, (t.y * v.x + b.y * v.y) + n.y * v.z,
            (t.z * v.x + b.z * v.y) + n.z * v.z);
}

__device__ __forceinline__ float glsl_max(float x, float y) { return x < y ? y : x; }

// normalize(v) = v / length(v): three IEEE quotients sharing one correctly
// rounded reciprocal.
__device__ __forceinline__ Float3 normalize3(Float3 l) {
  float len = sqrtf((l.x * l.x + l.y * l.y) + l.z * l.z);
  float r = 1.0f / len;
  return f3(agb_div_rcp(l.x, len, r), agb_div_rcp(l.y, len, r), agb_div_rcp(l.z, len, r));
}

// rng() of PreFilterEnvMap.comp:38-44: the seed advances by one per call, so
// draw k (1-based) is a pure function of seed0 + k.
__device__ __forceinline__ uint32_t hash_bits(uint32_t sx, uint32_t sy) {
  uint32_t qx = 1103515245u * ((sx >> 1u) ^ sy);
  uint32_t qy = 1103515245u * ((sy >> 1u) ^ sx);
  return 1103515245u * (qx ^ (qy >> 3u));
}

__device__ __forceinline__ float hash_float(uint32_t n) {
  return __uint2float_rn(n) * (1.0f / 4294967296.0f);
}

__device__ __forceinline__ void hammersley(int i, int n, float& x, float& y) {
  x = (float)i / (float)n;
  y = __uint2float_rn(__brev((uint32_t)i)) * (1.0f / 4294967296.0f);
}

// sampleGGX (PreFilterEnvMap.comp:84-92) with xi supplied.
__device__ __forceinline__ Float3 sample_ggx(float xi_x, float xi_y, float a2) {
  float phi = 2.0f * kPi * xi_x;
  float cos_t = sqrtf((1.0f - xi_y) / (1.0f + (a2 - 1.0f) * xi_y));
  float sin_t = sqrtf(1.0f - cos_t * cos_t);
  float sp, cp;
  agb_sincos(phi, &sp, &cp);
  return f3(cp * sin_t, sp * sin_t, cos_t);
}

// distributionGGX (PreFilterEnvMap.comp:78-82).
__device__ __forceinline__ float distribution_ggx(float ndoth, float a2) {
  float denom = (ndoth * ndoth * (a2 - 1.0f) + 1.0f);
  return a2 / (kPi * denom * denom);
}

}  // namespace ibl
