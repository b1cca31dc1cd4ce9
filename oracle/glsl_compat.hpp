// glsl_compat.hpp -- just enough GLSL 450 for three compute shaders of the
// reference (Shaders/IBL_Precompute/GenIrradianceMap.comp, PreFilterEnvMap.comp
// and Shaders/SSRGlossyConvolve.comp) to compile unmodified-in-substance as C++
// after the mechanical rewrite done by oracle/make_ref.py.  TEST INFRASTRUCTURE
// ONLY.
//
// Semantics chosen where GLSL leaves them to the implementation:
//  * transcendental built-ins -> glsl_builtins.h (fixed, portable);
//  * sqrt and division -> IEEE-754 single (correctly rounded);
//  * max(x, y) = x < y ? y : x (GLSL spec 8.3);
//  * length/normalize/dot sum left to right; mat3*vec3 = c0*v.x + c1*v.y + c2*v.z;
//  * textureLod -> the Vulkan-spec trilinear filter (REPEAT, LINEAR, LINEAR)
//    over a vkCmdBlitImage-equivalent mip chain, both written again here
//    independently of oracle/ibl_oracle.c;
//  * bindless heap textures (SAMPLER2D / IMAGE2D_W of Bindless/GlobalHeap.glsl)
//    -> one-level RGBA16F views sampled LINEAR with CLAMP_TO_EDGE (the
//    reference's default SamplerOptions, Include/Althea/Sampler.h:16-29), and
//    RGBA16F stores rounded to nearest even; the binary16 conversions are
//    written from the format's definition, independently of oracle/ssr_oracle.c.
// Build with -ffp-contract=off so no multiply-add is fused.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

#include "../althea_gb300/csrc/glsl_builtins.h"

namespace glslc {

typedef uint32_t uint;
struct uvec2;
struct ivec2 {
  int x, y;
  ivec2() : x(0), y(0) {}
  ivec2(int a, int b) : x(a), y(b) {}
  explicit ivec2(const uvec2& u);
};
struct vec2 {
  float x, y;
  vec2() : x(0), y(0) {}
  explicit vec2(float s) : x(s), y(s) {}
  vec2(float a, float b) : x(a), y(b) {}
  explicit vec2(const ivec2& i) : x((float)i.x), y((float)i.y) {}
};
struct vec3 {
  float x, y, z;
  vec3() : x(0), y(0), z(0) {}
  explicit vec3(float s) : x(s), y(s), z(s) {}
  vec3(float a, float b, float c) : x(a), y(b), z(c) {}
  vec2 xz() const { return vec2(x, z); }
  vec2 xy() const { return vec2(x, y); }
  vec3& operator+=(const vec3& o) {
    x = x + o.x;
    y = y + o.y;
    z = z + o.z;
    return *this;
  }
};
struct vec4 {
  float x, y, z, w;
  vec4() : x(0), y(0), z(0), w(0) {}
  explicit vec4(float s) : x(s), y(s), z(s), w(s) {}
  vec4(float a, float b, float c, float d) : x(a), y(b), z(c), w(d) {}
  vec4(const vec3& v, float d) : x(v.x), y(v.y), z(v.z), w(d) {}
  vec3 rgb() const { return vec3(x, y, z); }
  vec4& operator+=(const vec4& o) {
    x = x + o.x;
    y = y + o.y;
    z = z + o.z;
    w = w + o.w;
    return *this;
  }
};
struct uvec2 {
  uint32_t x, y;
  uvec2() : x(0), y(0) {}
  explicit uvec2(uint32_t s) : x(s), y(s) {}
  uvec2(uint32_t a, uint32_t b) : x(a), y(b) {}
  uvec2 yx() const { return uvec2(y, x); }
  uvec2& operator+=(const uvec2& o) {
    x += o.x;
    y += o.y;
    return *this;
  }
};
struct uvec3 {
  uint32_t x, y, z;
  uvec2 xy() const { return uvec2(x, y); }
};
inline ivec2::ivec2(const uvec2& u) : x((int)u.x), y((int)u.y) {}

struct mat3 {
  vec3 c0, c1, c2;
  mat3(const vec3& a, const vec3& b, const vec3& c) : c0(a), c1(b), c2(c) {}
};

inline uvec2 operator>>(const uvec2& a, uint32_t s) { return uvec2(a.x >> s, a.y >> s); }
inline uvec2 operator^(const uvec2& a, const uvec2& b) { return uvec2(a.x ^ b.x, a.y ^ b.y); }
inline uvec2 operator*(uint32_t s, const uvec2& a) { return uvec2(s * a.x, s * a.y); }

inline vec2 operator*(float s, const vec2& a) { return vec2(s * a.x, s * a.y); }
inline vec2 operator-(const vec2& a, float s) { return vec2(a.x - s, a.y - s); }
inline vec2 operator/(const vec2& a, const vec2& b) { return vec2(a.x / b.x, a.y / b.y); }
inline vec2 operator/(const vec2& a, float s) { return vec2(a.x / s, a.y / s); }
inline vec2 operator*(const vec2& a, const vec2& b) { return vec2(a.x * b.x, a.y * b.y); }
inline vec2 operator+(const vec2& a, const vec2& b) { return vec2(a.x + b.x, a.y + b.y); }
inline vec2 operator-(const vec2& a, const vec2& b) { return vec2(a.x - b.x, a.y - b.y); }
inline vec4 operator*(const vec4& a, float s) { return vec4(a.x * s, a.y * s, a.z * s, a.w * s); }

inline vec3 operator+(const vec3& a, const vec3& b) { return vec3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline vec3 operator-(const vec3& a, const vec3& b) { return vec3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline vec3 operator*(const vec3& a, float s) { return vec3(a.x * s, a.y * s, a.z * s); }
inline vec3 operator*(float s, const vec3& a) { return vec3(s * a.x, s * a.y, s * a.z); }
inline vec3 operator/(const vec3& a, float s) { return vec3(a.x / s, a.y / s, a.z / s); }
inline vec3 operator*(const mat3& m, const vec3& v) {
  return vec3((m.c0.x * v.x + m.c1.x * v.y) + m.c2.x * v.z,
              (m.c0.y * v.x + m.c1.y * v.y) + m.c2.y * v.z,
              (m.c0.z * v.x + m.c1.z * v.y) + m.c2.z * v.z);
}

inline float abs(float x) { return agb_abs(x); }
inline float sqrt(float x) { return sqrtf(x); }
inline float cos(float x) { return agb_cos(x); }
inline float sin(float x) { return agb_sin(x); }
inline float atan(float x) { return agb_atan(x); }
inline float atan(float y, float x) { return agb_atan2(y, x); }
inline float log2(float x) { return agb_log2(x); }
inline float max(float x, float y) { return x < y ? y : x; }
inline float min(float x, float y) { return y < x ? y : x; }
inline float clamp(float x, float lo, float hi) { return min(max(x, lo), hi); }
inline float dot(const vec3& a, const vec3& b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
inline float length(const vec2& a) { return sqrtf(a.x * a.x + a.y * a.y); }
inline float length(const vec3& a) { return sqrtf(dot(a, a)); }
inline vec3 normalize(const vec3& a) { return a / length(a); }
inline vec3 cross(const vec3& a, const vec3& b) {
  return vec3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}

// ---- resources -------------------------------------------------------------
struct sampler2D {};
struct image2D {};

struct Resources {
  const float* chain = nullptr;  // RGBA32F levels back to back
  int w = 0, h = 0, levels = 0;
  float* out = nullptr;  // RGBA32F output image
  int ow = 0, oh = 0;
};
extern Resources g_res;
extern thread_local uvec3 gl_GlobalInvocationID;

inline void level_dims(int l, int* lw, int* lh) {
  int a = g_res.w >> l, b = g_res.h >> l;
  *lw = a < 1 ? 1 : a;
  *lh = b < 1 ? 1 : b;
}
inline const float* level_ptr(int l) {
  size_t off = 0;
  for (int i = 0; i < l; ++i) {
    int lw, lh;
    level_dims(i, &lw, &lh);
    off += (size_t)lw * lh;
  }
  return g_res.chain + 4 * off;
}
inline int wrap_repeat(int i, int n) {
  int r = i % n;
  return r < 0 ? r + n : r;
}
inline vec4 fetch(const float* img, int lw, int i, int j) {
  const float* p = img + 4 * ((size_t)j * lw + i);
  return vec4(p[0], p[1], p[2], p[3]);
}
inline vec4 bilinear(const vec4& t00, const vec4& t10, const vec4& t01, const vec4& t11,
                     float a, float b) {
  float w00 = (1.0f - a) * (1.0f - b), w10 = a * (1.0f - b);
  float w01 = (1.0f - a) * b, w11 = a * b;
  return vec4(((w00 * t00.x + w10 * t10.x) + w01 * t01.x) + w11 * t11.x,
              ((w00 * t00.y + w10 * t10.y) + w01 * t01.y) + w11 * t11.y,
              ((w00 * t00.z + w10 * t10.z) + w01 * t01.z) + w11 * t11.z,
              ((w00 * t00.w + w10 * t10.w) + w01 * t01.w) + w11 * t11.w);
}
inline vec4 sample_level(int l, const vec2& uv) {
  int lw, lh;
  level_dims(l, &lw, &lh);
  const float* img = level_ptr(l);
  float x = uv.x * (float)lw - 0.5f, y = uv.y * (float)lh - 0.5f;
  float fx = floorf(x), fy = floorf(y);
  int i0 = wrap_repeat((int)fx, lw), i1 = wrap_repeat((int)fx + 1, lw);
  int j0 = wrap_repeat((int)fy, lh), j1 = wrap_repeat((int)fy + 1, lh);
  return bilinear(fetch(img, lw, i0, j0), fetch(img, lw, i1, j0), fetch(img, lw, i0, j1),
                  fetch(img, lw, i1, j1), x - fx, y - fy);
}
inline vec4 textureLod(const sampler2D&, const vec2& uv, float lod) {
  int q = g_res.levels - 1;
  float lam = lod < 0.0f ? 0.0f : (lod > (float)q ? (float)q : lod);
  float fl = floorf(lam);
  int l0 = (int)fl;
  float d = lam - fl;
  vec4 lo = sample_level(l0, uv);
  if (!(d > 0.0f)) return lo;
  vec4 hi = sample_level(l0 + 1 > q ? q : l0 + 1, uv);
  return vec4((1.0f - d) * lo.x + d * hi.x, (1.0f - d) * lo.y + d * hi.y,
              (1.0f - d) * lo.z + d * hi.z, (1.0f - d) * lo.w + d * hi.w);
}
inline void imageStore(const image2D&, const ivec2& p, const vec4& c) {
  float* o = g_res.out + 4 * ((size_t)p.y * g_res.ow + p.x);
  o[0] = c.x;
  o[1] = c.y;
  o[2] = c.z;
  o[3] = c.w;
}

// ---- bindless heap of one-level RGBA16F views (SSRGlossyConvolve) ---------
struct HalfView {
  const uint16_t* src = nullptr;  // sampled view: 4 halfs per texel, row-major
  uint16_t* dst = nullptr;        // storage view
  int w = 0, h = 0;
};
extern HalfView g_heap_tex[4], g_heap_img[4];
struct HeapTexture { uint idx; };
struct HeapImage { uint idx; };
struct SamplerHeap {
  HeapTexture operator[](uint i) const { return HeapTexture{i}; }
};
struct ImageHeap {
  HeapImage operator[](uint i) const { return HeapImage{i}; }
};
#define SAMPLER2D(NAME) glslc::SamplerHeap NAME
#define IMAGE2D_W(NAME) glslc::ImageHeap NAME

// binary16 -> binary32: (-1)^s * 2^(e-15) * (1 + m/1024), subnormals 2^-14 * m/1024.
inline float half_value(uint16_t hbits) {
  int e = (hbits >> 10) & 31, m = hbits & 1023;
  float mag;
  if (e == 31)
    mag = m ? NAN : INFINITY;
  else if (e == 0)
    mag = ldexpf((float)m, -24);
  else
    mag = ldexpf((float)(1024 + m), e - 25);
  return (hbits & 0x8000) ? -mag : mag;
}
// binary32 -> binary16, round to nearest even: scale the magnitude so the
// kept bits are the integer part (exact, a power of two) and round that with
// nearbyintf in the default round-to-nearest-even mode.
inline uint16_t half_bits(float f) {
  uint16_t sign = signbit(f) ? 0x8000 : 0;
  float a = fabsf(f);
  if (isnan(a)) return (uint16_t)(sign | 0x7e00);
  if (a >= 65520.0f) return (uint16_t)(sign | 0x7c00);  // ties above 65504 round to inf
  if (a < ldexpf(1.0f, -14)) return (uint16_t)(sign | (uint16_t)nearbyintf(ldexpf(a, 24)));
  int k;
  frexpf(a, &k);  // a in [2^(k-1), 2^k)
  int e = k - 1;
  int q = (int)nearbyintf(ldexpf(a, 10 - e));  // 1024..2048
  if (q == 2048) {
    q = 1024;
    e += 1;
  }
  return (uint16_t)(sign | ((e + 15) << 10) | (q - 1024));
}
inline vec4 fetch_half(const HalfView& v, int i, int j) {
  const uint16_t* p = v.src + 4 * ((size_t)j * v.w + i);
  return vec4(half_value(p[0]), half_value(p[1]), half_value(p[2]), half_value(p[3]));
}
inline int clamp_to_edge(int i, int n) { return i < 0 ? 0 : (i >= n ? n - 1 : i); }
// The view has one level and the sampler minLod = maxLod = 0: level 0, LINEAR.
inline vec4 textureLod(const HeapTexture& t, const vec2& uv, float) {
  const HalfView& v = g_heap_tex[t.idx];
  float x = uv.x * (float)v.w - 0.5f, y = uv.y * (float)v.h - 0.5f;
  float fx = floorf(x), fy = floorf(y);
  int i0 = clamp_to_edge((int)fx, v.w), i1 = clamp_to_edge((int)fx + 1, v.w);
  int j0 = clamp_to_edge((int)fy, v.h), j1 = clamp_to_edge((int)fy + 1, v.h);
  return bilinear(fetch_half(v, i0, j0), fetch_half(v, i1, j0), fetch_half(v, i0, j1),
                  fetch_half(v, i1, j1), x - fx, y - fy);
}
inline void imageStore(const HeapImage& im, const ivec2& p, const vec4& c) {
  const HalfView& v = g_heap_img[im.idx];
  uint16_t* o = v.dst + 4 * ((size_t)p.y * v.w + p.x);
  o[0] = half_bits(c.x);
  o[1] = half_bits(c.y);
  o[2] = half_bits(c.z);
  o[3] = half_bits(c.w);
}

// Sample-index counter for the Hammersley variant of sampleGGX's xi source.
extern thread_local int g_sample_index;
extern int g_sample_count;
inline vec2 hammersley_next() {
  uint32_t i = (uint32_t)g_sample_index++;
  uint32_t v = i;
  v = ((v >> 1) & 0x55555555u) | ((v & 0x55555555u) << 1);
  v = ((v >> 2) & 0x33333333u) | ((v & 0x33333333u) << 2);
  v = ((v >> 4) & 0x0f0f0f0fu) | ((v & 0x0f0f0f0fu) << 4);
  v = ((v >> 8) & 0x00ff00ffu) | ((v & 0x00ff00ffu) << 8);
  v = (v >> 16) | (v << 16);
  return vec2((float)i / (float)g_sample_count, (float)v * (1.0f / 4294967296.0f));
}

}  // namespace glslc

// Names a shader namespace pulls in; using-declarations hide <math.h>'s
// overloads of the same names inside the shader's namespace.
#define GLSLC_USING                                                            \
  using glslc::uint;                                                           \
  using glslc::vec2;                                                           \
  using glslc::vec3;                                                           \
  using glslc::vec4;                                                           \
  using glslc::uvec2;                                                          \
  using glslc::ivec2;                                                          \
  using glslc::mat3;                                                           \
  using glslc::sampler2D;                                                      \
  using glslc::image2D;                                                        \
  using glslc::abs;                                                            \
  using glslc::sqrt;                                                           \
  using glslc::cos;                                                            \
  using glslc::sin;                                                            \
  using glslc::atan;                                                           \
  using glslc::log2;                                                           \
  using glslc::max;                                                            \
  using glslc::clamp;                                                          \
  using glslc::dot;                                                            \
  using glslc::length;                                                         \
  using glslc::normalize;                                                      \
  using glslc::cross;                                                          \
  using glslc::textureLod;                                                     \
  using glslc::imageStore;                                                     \
  using glslc::gl_GlobalInvocationID;
