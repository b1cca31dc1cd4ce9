/*
 * glsl_builtins.h -- one fixed implementation of the GLSL transcendental
 * built-ins used by the IBL precompute shaders (sin, cos, atan, atan(y,x),
 * log2), compiled identically as C (host oracle) and CUDA (device kernels).
 *
 * Why this exists.  GLSL leaves the precision of these built-ins to the
 * implementation.  The reference shaders (Shaders/IBL_Precompute/
 * PreFilterEnvMap.comp:87-91,106-107,131-134,161 and GenIrradianceMap.comp:
 * 86-87,111-114,124-134) map a texel to a direction and back to texture
 * coordinates; at roughness 0 one unit in the last place of u moves a
 * bilinear weight by about W*6e-8 texels, i.e. ~2e-4 relative on high-
 * contrast maps -- larger than the 1e-4 parity bar.  Host libm and CUDA's
 * libdevice differ by 1-3 ulp, so parity at roughness 0 is only meaningful
 * when both sides use the same implementation.  Every function here uses
 * only IEEE-754 single operations (+ - * / sqrt, fmaf, rintf, bit moves),
 * so a C build with -ffp-contract=off and a CUDA build with -fmad=false
 * produce bit-identical results.
 *
 * Methods (textbook, not any vendor's library):
 *   sin/cos : Cody & Waite (1980) additive range reduction by pi/2 with a
 *             three-part constant, then the Taylor series of sin (to x^11)
 *             and cos (to x^12) on [-pi/4, pi/4]; truncation < 1e-11.
 *   atan    : argument reduction x -> 1/x for |x|>1 and
 *             atan t = pi/6 + atan((sqrt3*t - 1)/(t + sqrt3)) for t > 2-sqrt3,
 *             then the Taylor series to u^15 (|u| <= 0.268, truncation ~4e-11).
 *   atan2   : quadrant logic of C99 atan2 on top of atan.
 *   log2    : x = m*2^e with m in [sqrt(1/2), sqrt(2)),
 *             log2 m = (2/ln 2) * atanh(s), s = (m-1)/(m+1), series to s^13.
 * Constants are the float roundings of pi/2, pi/6 and friends split into
 * hi/mid/lo parts; they follow from the mathematics alone.
 * Accuracy (checked in tests against double-precision libm): <= 3 ulp.
 */
#ifndef ALTHEA_GLSL_BUILTINS_H
#define ALTHEA_GLSL_BUILTINS_H

#include <stdint.h>

#if defined(__CUDACC__)
#define AGB_FN static __host__ __device__ __forceinline__
#define AGB_FMA(a, b, c) fmaf((a), (b), (c))
#define AGB_RINT(x) rintf(x)
#define AGB_SQRT(x) sqrtf(x)
#else
#include <math.h>
#include <string.h>
#define AGB_FN static inline
#define AGB_FMA(a, b, c) fmaf((a), (b), (c))
#define AGB_RINT(x) rintf(x)
#define AGB_SQRT(x) sqrtf(x)
#endif

AGB_FN uint32_t agb_bits(float x) {
#if defined(__CUDA_ARCH__)
  return __float_as_uint(x);
#else
  uint32_t u;
  memcpy(&u, &x, 4);
  return u;
#endif
}

AGB_FN float agb_float(uint32_t u) {
#if defined(__CUDA_ARCH__)
  return __uint_as_float(u);
#else
  float x;
  memcpy(&x, &u, 4);
  return x;
#endif
}

AGB_FN float agb_abs(float x) { return agb_float(agb_bits(x) & 0x7fffffffu); }
AGB_FN float agb_copysign(float mag, float sgn) {
  return agb_float((agb_bits(mag) & 0x7fffffffu) | (agb_bits(sgn) & 0x80000000u));
}

/* pi/2, pi and pi/6 as hi + mid + lo float parts (hi carries 24 bits). */
#define AGB_PIO2_HI 0x1.921fb6p+0f
#define AGB_PIO2_MID -0x1.777a5cp-25f
#define AGB_PIO2_LO -0x1.ee59dap-50f
#define AGB_PI_HI 0x1.921fb6p+1f
#define AGB_PI_MID -0x1.777a5cp-24f
#define AGB_PI6_HI 0x1.0c1524p-1f
#define AGB_PI6_MID -0x1.f4a326p-27f
#define AGB_TWO_OVER_PI 0x1.45f306p-1f
#define AGB_TWO_OVER_LN2 0x1.715476p+1f
#define AGB_SQRT3 0x1.bb67aep+0f
#define AGB_TWO_MINUS_SQRT3 0x1.126146p-2f
#define AGB_SQRT2 0x1.6a09e6p+0f

/* Taylor polynomials on the reduced interval |r| <= pi/4 (+ a little). */
AGB_FN float agb_sin_poly(float r) {
  float r2 = r * r;
  float p = AGB_FMA(r2, -2.50521083854417188e-08f, 2.75573192239858907e-06f);
  p = AGB_FMA(r2, p, -1.98412698412698413e-04f);
  p = AGB_FMA(r2, p, 8.33333333333333333e-03f);
  p = AGB_FMA(r2, p, -1.66666666666666667e-01f);
  return AGB_FMA(r * r2, p, r);
}

AGB_FN float agb_cos_poly(float r) {
  float r2 = r * r;
  float p = AGB_FMA(r2, 2.08767569878680990e-09f, -2.75573192239858907e-07f);
  p = AGB_FMA(r2, p, 2.48015873015873016e-05f);
  p = AGB_FMA(r2, p, -1.38888888888888889e-03f);
  p = AGB_FMA(r2, p, 4.16666666666666667e-02f);
  p = AGB_FMA(r2, p, -0.5f);
  return AGB_FMA(r2, p, 1.0f);
}

/* Reduce x to r in [-pi/4, pi/4] with x = k*pi/2 + r; returns k mod 4.
 * Valid (error well below 1 ulp of r) for |x| up to ~1e4. */
AGB_FN int agb_reduce_pio2(float x, float* r_out) {
  float k = AGB_RINT(x * AGB_TWO_OVER_PI);
  float r = AGB_FMA(-k, AGB_PIO2_HI, x);
  r = AGB_FMA(-k, AGB_PIO2_MID, r);
  r = AGB_FMA(-k, AGB_PIO2_LO, r);
  *r_out = r;
  return ((int)k) & 3;
}

AGB_FN float agb_sin(float x) {
  float r;
  int q = agb_reduce_pio2(x, &r);
  float s = agb_sin_poly(r), c = agb_cos_poly(r);
  float v = (q & 1) ? c : s;
  return (q & 2) ? -v : v;
}

AGB_FN float agb_cos(float x) {
  float r;
  int q = agb_reduce_pio2(x, &r);
  float s = agb_sin_poly(r), c = agb_cos_poly(r);
  float v = (q & 1) ? s : c;
  return ((q + 1) & 2) ? -v : v;
}

/* Both at once: one reduction, the same results as agb_sin / agb_cos. */
AGB_FN void agb_sincos(float x, float* sn, float* cs) {
  float r;
  int q = agb_reduce_pio2(x, &r);
  float s = agb_sin_poly(r), c = agb_cos_poly(r);
  float vs = (q & 1) ? c : s;
  float vc = (q & 1) ? s : c;
  *sn = (q & 2) ? -vs : vs;
  *cs = ((q + 1) & 2) ? -vc : vc;
}

/* atan on t in [0, 1]. */
AGB_FN float agb_atan01(float t) {
  int red = t > AGB_TWO_MINUS_SQRT3;
  float u = red ? AGB_FMA(t, AGB_SQRT3, -1.0f) / (t + AGB_SQRT3) : t;
  float u2 = u * u;
  float p = AGB_FMA(u2, -6.66666666666666667e-02f, 7.69230769230769231e-02f);
  p = AGB_FMA(u2, p, -9.09090909090909091e-02f);
  p = AGB_FMA(u2, p, 1.11111111111111111e-01f);
  p = AGB_FMA(u2, p, -1.42857142857142857e-01f);
  p = AGB_FMA(u2, p, 2.00000000000000000e-01f);
  p = AGB_FMA(u2, p, -3.33333333333333333e-01f);
  float a = AGB_FMA(u * u2, p, u);
  return red ? (a + AGB_PI6_MID) + AGB_PI6_HI : a;
}

/* GLSL atan(y_over_x): range (-pi/2, pi/2). */
AGB_FN float agb_atan(float x) {
  float t = agb_abs(x);
  if (t != t) return x; /* NaN */
  int inv = t > 1.0f;
  float a = agb_atan01(inv ? 1.0f / t : t);
  if (inv) a = (AGB_PIO2_MID - a) + AGB_PIO2_HI;
  return agb_copysign(a, x);
}

/* GLSL atan(y, x): range [-pi, pi], C99 conventions for signed zeros. */
AGB_FN float agb_atan2(float y, float x) {
  float ax = agb_abs(x), ay = agb_abs(y);
  if (ax != ax || ay != ay) return x + y; /* NaN */
  float a;
  if (ax == 0.0f && ay == 0.0f) {
    a = 0.0f;
  } else {
    int swap = ay > ax;
    a = agb_atan01(swap ? ax / ay : ay / ax);
    if (swap) a = (AGB_PIO2_MID - a) + AGB_PIO2_HI;
  }
  if (agb_bits(x) & 0x80000000u) a = (AGB_PI_MID - a) + AGB_PI_HI;
  return agb_copysign(a, y);
}

/* log2 of a positive normal finite x (the common case of agb_log2). */
AGB_FN float agb_log2_core(uint32_t b, int e) {
  e += (int)(b >> 23) - 127;
  float m = agb_float((b & 0x007fffffu) | 0x3f800000u);
  if (m > AGB_SQRT2) {
    m = m * 0.5f;
    e += 1;
  }
  float s = (m - 1.0f) / (m + 1.0f);
  float s2 = s * s;
  float p = AGB_FMA(s2, 7.69230769230769231e-02f, 9.09090909090909091e-02f);
  p = AGB_FMA(s2, p, 1.11111111111111111e-01f);
  p = AGB_FMA(s2, p, 1.42857142857142857e-01f);
  p = AGB_FMA(s2, p, 2.00000000000000000e-01f);
  p = AGB_FMA(s2, p, 3.33333333333333333e-01f);
  float l = AGB_FMA(s * s2, p, s) * AGB_TWO_OVER_LN2;
  return (float)e + l;
}

/* GLSL log2: -inf at 0, NaN below 0, +inf at +inf. */
AGB_FN float agb_log2(float x) {
  uint32_t b = agb_bits(x);
  if (b - 0x00800000u < 0x7f000000u) return agb_log2_core(b, 0); /* positive normal */
  if (x != x) return x;
  if (x < 0.0f) return agb_float(0x7fc00000u);
  if (x == 0.0f) return agb_float(0xff800000u);
  if (b == 0x7f800000u) return x;
  /* positive subnormal: scale by 2^23 */
  return agb_log2_core(agb_bits(x * 8388608.0f), -23);
}

/* a / b correctly rounded, given r = the correctly rounded 1/b (Markstein's
 * theorem: q0 = a*r is within one ulp of a/b and the fma-computed residual
 * a - q0*b is exact, so q0 + residual*r rounds to the IEEE quotient; zero
 * numerators keep their sign).  Valid while a/b neither overflows nor
 * underflows.  Saves the full division where the denominator is shared or
 * constant. */
AGB_FN float agb_div_rcp(float a, float b, float r) {
  float q0 = a * r;
  float e = AGB_FMA(-q0, b, a);
  float q = AGB_FMA(e, r, q0);
  return a == 0.0f ? q0 : q;
}

/* Split-sum BRDF LUT (Karis 2013, IntegrateBRDF): one Hammersley sample's
 * terms for a texel with view vector (vx, 0, vz), given the sample's half
 * vector (hx, 0-plane, hz), 1 / NoH, omk = 1 - k, k = alpha / 2 and
 * gv = G1(V) / NoV: adds (1 - Fc) G_vis to *sum_a and Fc G_vis to *sum_b,
 * G_vis = G1(L) G1(V) VoH / (NoH NoV), Fc = (1 - VoH)^5.  Every product-sum
 * is one explicit fma and 1 / (NoL (1 - k) + k) a correctly rounded
 * reciprocal, so the LUT kernels and the CPU oracle, which both call this,
 * compute the same bits. */
AGB_FN void agb_lut_sample(float vx, float vz, float hx, float hz, float rnoh, float omk, float k,
                           float gv, float* sum_a, float* sum_b) {
  const float vdh = AGB_FMA(vx, hx, vz * hz);
  const float lz = AGB_FMA(2.0f * vdh, hz, -vz);
  const float nol = lz > 0.0f ? (lz < 1.0f ? lz : 1.0f) : 0.0f;
  const float voh = vdh > 0.0f ? (vdh < 1.0f ? vdh : 1.0f) : 0.0f;
  if (nol > 0.0f) {
    const float g1l = nol * (1.0f / AGB_FMA(nol, omk, k));
    const float g_vis = ((g1l * gv) * voh) * rnoh;
    const float tt = 1.0f - voh;
    const float t2 = tt * tt;
    const float fc = t2 * t2 * tt;
    *sum_a = AGB_FMA(1.0f - fc, g_vis, *sum_a);
    *sum_b = AGB_FMA(fc, g_vis, *sum_b);
  }
}

/* Correctly rounded reciprocals of 2*pi and pi as single-precision values
 * (1 / 6.2831855f and 1 / 3.1415927f). */
#define AGB_RCP_TWO_PI_F 0x1.45f306p-3f
#define AGB_RCP_PI_F 0x1.45f306p-2f

#endif /* ALTHEA_GLSL_BUILTINS_H */
