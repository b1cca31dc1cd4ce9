/*
 * ssr_oracle.c -- CPU oracle for the reflection-buffer glossy convolution.
 * TEST INFRASTRUCTURE ONLY: the tests and the CPU-baseline leg of the bench
 * call it to check the product's results; nothing in the product library
 * links or calls it.
 *
 * Restates Shaders/SSRGlossyConvolve.comp:25-53 as dispatched by
 * ReflectionBuffer::convolveReflectionBuffer (Src/ReflectionBuffer.cpp:
 * 163-275): for mip levels 1..mips-1 of an RGBA16F reflection buffer
 * (Src/ReflectionBuffer.cpp:28-36), a 7-tap Gaussian along `direction`
 * (vertical for odd levels, horizontal for even ones) reads level l-1 through
 * a CLAMP_TO_EDGE / LINEAR sampler of that one level (Src/ReflectionBuffer.cpp:
 * 62-64, default SamplerOptions) at uv = texelPos / (w_l, h_l), offsets
 * divided by w_l in both directions, and stores level l as RGBA16F.
 *
 * Sampling follows the Vulkan spec in FP32 with the bilinear combination
 * ((w00 t00 + w10 t10) + w01 t01) + w11 t11; half <-> float conversions are
 * IEEE 754 binary16 with round-to-nearest-even (written from the format's
 * definition below).  Images: row-major, 4 halfs per texel, every level
 * packed back to back, level 0 first.
 */
#include <math.h>
#include <stdint.h>
#include <string.h>

#include "ibl_oracle.h"

float oracle_half_to_float(uint16_t h) {
  uint32_t sign = (uint32_t)(h >> 15) << 31;
  int exp = (h >> 10) & 0x1f;
  uint32_t man = h & 0x3ff;
  uint32_t bits;
  if (exp == 0) {
    if (man == 0) {
      bits = sign;
    } else {  /* subnormal: man * 2^-24, exact in binary32 */
      float f = (float)man * (1.0f / 16777216.0f);
      memcpy(&bits, &f, 4);
      bits |= sign;
    }
  } else if (exp == 31) {
    bits = sign | 0x7f800000u | (man << 13);
  } else {
    bits = sign | ((uint32_t)(exp - 15 + 127) << 23) | (man << 13);
  }
  float f;
  memcpy(&f, &bits, 4);
  return f;
}

uint16_t oracle_float_to_half(float f) {
  uint32_t x;
  memcpy(&x, &f, 4);
  uint16_t sign = (uint16_t)((x >> 16) & 0x8000);
  uint32_t absx = x & 0x7fffffffu;
  if (absx >= 0x7f800000u) /* inf or nan */
    return (uint16_t)(sign | 0x7c00 | (absx > 0x7f800000u ? 0x200 : 0));
  int e = (int)(absx >> 23) - 127;
  if (e > 15) return (uint16_t)(sign | 0x7c00); /* overflow: inf */
  if (e >= -14) {
    /* normal half: 10 mantissa bits, round the 13 dropped bits to nearest even */
    uint32_t man = absx & 0x7fffff;
    uint32_t base = ((uint32_t)(e + 15) << 10) | (man >> 13);
    uint32_t rest = man & 0x1fff;
    if (rest > 0x1000 || (rest == 0x1000 && (base & 1))) base += 1; /* may carry into inf */
    return (uint16_t)(sign | base);
  }
  /* subnormal half: value / 2^-24 rounded to nearest even integer */
  if (e < -25) return sign; /* below half of the smallest subnormal */
  uint32_t man = (absx & 0x7fffff) | 0x800000;    /* 24-bit significand */
  int shift = -e - 14 + 13;                        /* bits dropped */
  uint32_t q = man >> shift;
  uint32_t rest = man & ((1u << shift) - 1);
  uint32_t half = 1u << (shift - 1);
  if (rest > half || (rest == half && (q & 1))) q += 1;
  return (uint16_t)(sign | q);
}

static int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

/* textureLod(level, uv, 0.0) with CLAMP_TO_EDGE, LINEAR */
static void sample_clamp(const uint16_t* img, int w, int h, float u, float v, float* out) {
  float x = u * (float)w - 0.5f;
  float y = v * (float)h - 0.5f;
  float fx = floorf(x), fy = floorf(y);
  float a = x - fx, b = y - fy;
  int i0 = clampi((int)fx, 0, w - 1), i1 = clampi((int)fx + 1, 0, w - 1);
  int j0 = clampi((int)fy, 0, h - 1), j1 = clampi((int)fy + 1, 0, h - 1);
  const uint16_t* t00 = img + 4 * ((size_t)j0 * w + i0);
  const uint16_t* t10 = img + 4 * ((size_t)j0 * w + i1);
  const uint16_t* t01 = img + 4 * ((size_t)j1 * w + i0);
  const uint16_t* t11 = img + 4 * ((size_t)j1 * w + i1);
  float w00 = (1.0f - a) * (1.0f - b);
  float w10 = a * (1.0f - b);
  float w01 = (1.0f - a) * b;
  float w11 = a * b;
  for (int c = 0; c < 4; ++c)
    out[c] = ((w00 * oracle_half_to_float(t00[c]) + w10 * oracle_half_to_float(t10[c])) +
              w01 * oracle_half_to_float(t01[c])) +
             w11 * oracle_half_to_float(t11[c]);
}

static int dim(int d, int l) {
  int v = d >> l;
  return v < 1 ? 1 : v;
}

size_t oracle_ssr_level_offset(int w, int h, int level) {
  size_t off = 0;
  for (int l = 0; l < level; ++l) off += (size_t)dim(w, l) * dim(h, l);
  return off;
}

/* The Gaussian's taps (SSRGlossyConvolve.comp:42-51). */
static const float kOff1 = 1.411764705882353f, kOff2 = 3.2941176470588234f,
                   kOff3 = 5.176470588235294f;
static const float kW0 = 0.1964825501511404f, kW1 = 0.2969069646728344f,
                   kW2 = 0.09447039785044732f, kW3 = 0.010381362401148057f;

void oracle_ssr_convolve(uint16_t* chain, int w, int h, int mips) {
  for (int l = 1; l < mips; ++l) {
    const int sw = dim(w, l - 1), sh = dim(h, l - 1), dw = dim(w, l), dh = dim(h, l);
    const uint16_t* src = chain + 4 * oracle_ssr_level_offset(w, h, l - 1);
    uint16_t* dst = chain + 4 * oracle_ssr_level_offset(w, h, l);
    const float dx = (l & 1) ? 0.0f : 1.0f, dy = (l & 1) ? 1.0f : 0.0f;
    const float res = (float)dw;
    const float o1x = kOff1 * dx, o1y = kOff1 * dy, o2x = kOff2 * dx, o2y = kOff2 * dy;
    const float o3x = kOff3 * dx, o3y = kOff3 * dy;
#pragma omp parallel for schedule(static)
    for (int y = 0; y < dh; ++y) {
      for (int x = 0; x < dw; ++x) {
        const float u = (float)x / (float)dw, v = (float)y / (float)dh;
        float s[4], acc[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        sample_clamp(src, sw, sh, u, v, s);
        for (int c = 0; c < 4; ++c) acc[c] = acc[c] + s[c] * kW0;
        sample_clamp(src, sw, sh, u + o1x / res, v + o1y / res, s);
        for (int c = 0; c < 4; ++c) acc[c] = acc[c] + s[c] * kW1;
        sample_clamp(src, sw, sh, u - o1x / res, v - o1y / res, s);
        for (int c = 0; c < 4; ++c) acc[c] = acc[c] + s[c] * kW1;
        sample_clamp(src, sw, sh, u + o2x / res, v + o2y / res, s);
        for (int c = 0; c < 4; ++c) acc[c] = acc[c] + s[c] * kW2;
        sample_clamp(src, sw, sh, u - o2x / res, v - o2y / res, s);
        for (int c = 0; c < 4; ++c) acc[c] = acc[c] + s[c] * kW2;
        sample_clamp(src, sw, sh, u + o3x / res, v + o3y / res, s);
        for (int c = 0; c < 4; ++c) acc[c] = acc[c] + s[c] * kW3;
        sample_clamp(src, sw, sh, u - o3x / res, v - o3y / res, s);
        for (int c = 0; c < 4; ++c) acc[c] = acc[c] + s[c] * kW3;
        for (int c = 0; c < 4; ++c) dst[4 * ((size_t)y * dw + x) + c] = oracle_float_to_half(acc[c]);
      }
    }
  }
}
